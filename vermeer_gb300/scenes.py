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
    """A soup of n_tris triangles: centroid uniform in [lo,hi)^3 (lo and hi
    scalars or per-axis triples), each vertex
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
def _cross32(a, b):
    """a x b in float32 scalar operations (the order libvmr's scene loader
    uses, so a scene written to .vnf and loaded back gets the same bits)."""
    f = np.float32
    a, b = np.asarray(a, f), np.asarray(b, f)
    return np.array([f(a[1] * b[2]) - f(a[2] * b[1]), f(a[2] * b[0]) - f(a[0] * b[2]),
                     f(a[0] * b[1]) - f(a[1] * b[0])], f)


def _norm32(a):
    """a * (1 / sqrt((x*x + y*y) + z*z)) in float32 (Vec3Normalize with an
    exact reciprocal square root)."""
    f = np.float32
    a = np.asarray(a, f)
    s = f(f(a[0] * a[0]) + f(a[1] * a[1]))
    s = f(s + f(a[2] * a[2]))
    r = f(f(1.0) / np.sqrt(s))
    return (a * r).astype(f)


def lookat_camera(eye, target, up, fov_deg: float, aspect: float, focal: float = 12.0) -> dict:
    """Camera node of type LookAt with one key (builtin/camera/camera.go:
    80-98, 109-193): W = normalize(From - To), u = normalize(Up x W),
    v = normalize(u x W), LocalToWorld = Translate(From) * Basis(u, v, W)
    (column-major), TanThetaFocal = tan(degToRad(Fov/2)) * Focal."""
    f32 = np.float32
    eye, target, up = (np.asarray(a, f32) for a in (eye, target, up))

    W = _norm32(eye - target)
    u = _norm32(_cross32(up, W))
    v = _norm32(_cross32(u, W))
    m = np.zeros(16, f32)
    m[0:3], m[4:7], m[8:11], m[12:15], m[15] = u, v, W, eye, 1.0
    pi = f32(3.14159265358)
    half = f32(fov_deg) / f32(2)
    tan = f32(np.tan(np.float64(half * pi / f32(180.0))))
    return dict(m=m, tan_theta_focal=f32(tan * f32(focal)), aspect=f32(aspect), focal=f32(focal), radius=f32(0),
                fov=f32(fov_deg))


def _tri_light_mesh(p0, p1, p2):
    """The emissive mesh a TriLight adds (builtin/light/triangle.go:537-565):
    three vertices with the face normal at each."""
    p = np.asarray([p0, p1, p2], np.float32)
    n = _norm32(_cross32(p[1] - p[0], p[2] - p[0]))
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


# -------------------------------------------------- extended-mode scenes ---
def _lattice(seed: int, ix, iy, iz) -> np.ndarray:
    """Value of the noise lattice at integer points: uniform in [-1, 1) from
    a SplitMix64 hash of (seed, ix, iy, iz)."""
    with np.errstate(over="ignore"):
        k = (np.asarray(ix, np.int64).astype(np.uint64) * np.uint64(0x8DA6B343)
             ^ np.asarray(iy, np.int64).astype(np.uint64) * np.uint64(0xD8163841)
             ^ np.asarray(iz, np.int64).astype(np.uint64) * np.uint64(0xCB1AB31F))
        z = np.uint64(seed) * _GOLD + k
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(40)).astype(np.float64) * (2.0 ** -23) - 1.0


def value_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """3-D value noise in [-1, 1): lattice values interpolated trilinearly
    with smoothstep weights."""
    f = np.floor(p)
    i = f.astype(np.int64)
    t = p - f
    w = t * t * (3.0 - 2.0 * t)
    out = np.zeros(p.shape[0])
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                c = _lattice(seed, i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz)
                wx = w[:, 0] if dx else 1 - w[:, 0]
                wy = w[:, 1] if dy else 1 - w[:, 1]
                wz = w[:, 2] if dz else 1 - w[:, 2]
                out += c * wx * wy * wz
    return out


def octasphere(center, radius: float, subdiv: int, displace: float = 0.0, seed: int = 0, freq: float = 4.0):
    """A sphere of 8*subdiv^2 triangles: each face of an octahedron split
    into a subdiv x subdiv triangle grid, vertices projected to the sphere and
    moved radially by radius*displace*value_noise(freq*unit_dir).  Wound
    so geometric normals point outward.  Returns (verts [3n,3] float32, idxp,
    normals [3n,3] float32 of the undisplaced sphere)."""
    n = subdiv
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    keep = ii + jj <= n
    gi, gj = ii[keep], jj[keep]
    index = -np.ones((n + 1, n + 1), np.int64)
    index[gi, gj] = np.arange(gi.size)
    tris = []
    for i in range(n):
        for j in range(n - i):
            tris.append((index[i, j], index[i + 1, j], index[i, j + 1]))
            if i + j < n - 1:
                tris.append((index[i + 1, j], index[i + 1, j + 1], index[i, j + 1]))
    tris = np.asarray(tris, np.int64)
    all_v = []
    for sx in (1, -1):
        for sy in (1, -1):
            for sz in (1, -1):
                A, B, C = np.array([sx, 0, 0.0]), np.array([0, sy, 0.0]), np.array([0, 0, sz * 1.0])
                if sx * sy * sz < 0:
                    B, C = C, B
                pts = (A[None] * (n - gi - gj)[:, None] + B[None] * gi[:, None] + C[None] * gj[:, None]) / n
                all_v.append(pts[tris].reshape(-1, 3))
    u = np.concatenate(all_v)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = radius * (1.0 + displace * value_noise(freq * u, seed)) if displace else np.full(u.shape[0], radius)
    verts = (np.asarray(center, np.float64)[None] + u * r[:, None]).astype(np.float32)
    return verts, np.arange(verts.shape[0], dtype=np.uint32), u.astype(np.float32)


def quad_light_mesh(p0, e1, e2):
    """The emissive mesh of a quad light: triangles (p0, p0+e1, p0+e1+e2)
    and (p0, p0+e1+e2, p0+e2), whose geometric normals point along e1 x e2."""
    p0, e1, e2 = (np.asarray(a, np.float32) for a in (p0, e1, e2))
    v = np.stack([p0, p0 + e1, p0 + e1 + e2, p0, p0 + e1 + e2, p0 + e2]).astype(np.float32)
    return v, np.arange(6, dtype=np.uint32)


def furnace(albedo: float = 0.5, env: float = 1.0, subdiv: int = 12) -> dict:
    """A flat-shaded (convex) tessellated unit sphere, Lambert albedo
    `albedo`, under a constant environment `env` and nothing else.  Every
    pixel that sees the sphere converges to albedo*env exactly (each bounce
    off a convex object sees only the environment), every other pixel to
    env."""
    v, i, _ = octasphere((0.0, 0.0, 0.0), 1.0, subdiv)
    shaders = [dict(diffuse_colour=(albedo, albedo, albedo), diffuse_strength=1.0, diffuse_roughness=0.0)]
    cam = lookat_camera((0.0, 0.0, -4.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0, 1.0)
    return dict(meshes=[dict(verts=v, idxp=i, shaders=[0])], shaders=shaders, lights=[], quad_lights=[],
                env=(env, env, env), camera=cam)


def sphere_grid(per_side: int = 16, subdiv: int = 32, seed: int = 3, width: int = 1920, height: int = 1080,
                env=(0.05, 0.06, 0.08)) -> dict:
    """The full-render configuration: per_side^2 noise-displaced spheres of
    8*subdiv^2 triangles (16x16 x 8,192 = 2,097,152 by default; radius 0.4,
    radial displacement 0.05 x value noise, seed 3) on a 40x40 ground plane,
    each with a mixed diffuse + GGX ShaderStd (diffuse colour uniform in
    [0.2, 0.8], weights 0.7/0.3, GGX roughness uniform in [0.05, 0.6],
    dielectric Fresnel with IOR 1.5, i.e. F0 = 0.04), four 2x2 quad lights of
    radiance 15 at height 8, a constant environment light, and a pinhole
    camera at the image's aspect."""
    meshes, shaders = [], []
    ns = per_side * per_side
    col = 0.2 + 0.6 * np.stack([uniform(seed, ns, 400 + k) for k in range(3)], axis=1)
    rough = 0.05 + 0.55 * uniform(seed, ns, 410)
    off = (per_side - 1) / 2.0
    for k in range(ns):
        gx, gz = k % per_side, k // per_side
        c = (gx - off, 0.4, gz - off)
        v, i, nrm = octasphere(c, 0.4, subdiv, displace=0.05, seed=seed * 1000 + k)
        shaders.append(dict(diffuse_colour=col[k], diffuse_strength=0.7, diffuse_roughness=0.0,
                            spec1_colour=(1.0, 1.0, 1.0), spec1_strength=0.3, spec1_roughness=float(rough[k]),
                            ior=1.5))
        meshes.append(dict(verts=v, idxp=i, shaders=[k]))
    g = 20.0
    gv = np.asarray([(-g, 0, -g), (-g, 0, g), (g, 0, g), (-g, 0, -g), (g, 0, g), (g, 0, -g)], np.float32)
    shaders.append(dict(diffuse_colour=(0.5, 0.5, 0.5), diffuse_strength=1.0, diffuse_roughness=0.0))
    meshes.append(dict(verts=gv, idxp=np.arange(6, dtype=np.uint32), shaders=[len(shaders) - 1]))
    light_shader = len(shaders)
    shaders.append(dict(emission_colour=(1.0, 1.0, 1.0), emission_strength=15.0, diffuse_colour=(0.0, 0.0, 0.0),
                        diffuse_strength=1.0, diffuse_roughness=0.0))
    quads = []
    for x, z in ((-4.0, -4.0), (4.0, -4.0), (-4.0, 4.0), (4.0, 4.0)):
        p0, e1, e2 = (x - 1.0, 8.0, z - 1.0), (2.0, 0.0, 0.0), (0.0, 0.0, 2.0)
        v, i = quad_light_mesh(p0, e1, e2)
        meshes.append(dict(verts=v, idxp=i, shaders=[light_shader]))
        quads.append(dict(p0=p0, e1=e1, e2=e2, shader=light_shader, mesh=len(meshes) - 1))
    cam = lookat_camera((0.0, 7.0, -16.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 45.0, width / height)
    return dict(meshes=meshes, shaders=shaders, lights=[], quad_lights=quads, env=tuple(env), camera=cam,
                width=width, height=height)


def small_room_ext(n_tris: int = 4096, seed: int = 1, env=(0.2, 0.25, 0.3)) -> dict:
    """The small room for the extended path tracer, with every light kind
    and lobe: the two TriLight panels, a 0.4 x 0.3 quad light recessed in the
    ceiling opening (radiance 5), a constant environment seen through the
    open side, and the soup's eight materials cycling through Lambert,
    OrenNayar (roughness 0.6), diffuse + GGX (roughness 0.3 and 0.7) and
    diffuse + mirror (Spec1Roughness 0)."""
    sc = small_room(n_tris, seed=seed)
    kinds = [
        dict(diffuse_roughness=0.0),
        dict(diffuse_roughness=0.6),
        dict(diffuse_roughness=0.0, spec1_colour=(1.0, 1.0, 1.0), spec1_strength=0.5, spec1_roughness=0.3, ior=1.5),
        dict(diffuse_roughness=0.0, spec1_colour=(0.9, 0.8, 0.6), spec1_strength=0.4, spec1_roughness=0.7,
             spec1_fresnel="Metal", spec1_fresnel_refl=(0.9, 0.6, 0.3)),
        dict(diffuse_roughness=0.0, spec1_colour=(1.0, 1.0, 1.0), spec1_strength=0.3, spec1_roughness=0.0, ior=1.5),
    ]
    for k, sid in enumerate(range(5, 13)):
        sc["shaders"][sid] = dict(sc["shaders"][sid], **kinds[k % len(kinds)])
    light_shader = len(sc["shaders"])
    sc["shaders"].append(dict(emission_colour=(1.0, 0.9, 0.8), emission_strength=5.0, diffuse_colour=(0.0, 0.0, 0.0),
                              diffuse_strength=1.0, diffuse_roughness=0.0))
    p0, e1, e2 = (-0.2, 1.15, -0.15), (0.4, 0.0, 0.0), (0.0, 0.0, 0.3)
    v, i = quad_light_mesh(p0, e1, e2)
    sc["meshes"].append(dict(verts=v, idxp=i, shaders=[light_shader]))
    sc["quad_lights"] = [dict(p0=p0, e1=e1, e2=e2, shader=light_shader, mesh=len(sc["meshes"]) - 1)]
    sc["env"] = tuple(env)
    return sc


def _box_faces(lo, hi, skip=()):
    """Triangles of the faces of an axis-aligned box (names: x0 x1 y0 y1 z0
    z1 for the faces at lo/hi of each axis), wound so normals point inward."""
    (x0, y0, z0), (x1, y1, z1) = lo, hi
    faces = {
        "y0": [(x0, y0, z0), (x0, y0, z1), (x1, y0, z1), (x1, y0, z0)],
        "y1": [(x0, y1, z0), (x1, y1, z0), (x1, y1, z1), (x0, y1, z1)],
        "z0": [(x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0)],
        "z1": [(x0, y0, z1), (x0, y1, z1), (x1, y1, z1), (x1, y0, z1)],
        "x0": [(x0, y0, z0), (x0, y1, z0), (x0, y1, z1), (x0, y0, z1)],
        "x1": [(x1, y0, z0), (x1, y0, z1), (x1, y1, z1), (x1, y1, z0)],
    }
    tris = []
    for name, (a, b, c, d) in faces.items():
        if name in skip:
            continue
        tris += [a, b, c, a, c, d]
    return tris


def slit_room(n_tris: int = 200_000, seed: int = 5, width: int = 1024, height: int = 1024) -> dict:
    """The path-guiding configuration: a 4 x 3 x 3 room (x in [-2, 2], y in
    [0, 3], z in [0, 3]) whose only light, a quad of radiance 200 facing the
    room, sits in a 0.4-deep chamber behind the x = 2 wall; the wall is cut
    by a horizontal slit 0.06 high across its whole depth (2% of its area),
    the only way the light reaches the room.  n_tris random diffuse
    triangles built like the small room's soup (centroids uniform in the
    room's interior, vertices at centroid + 0.02 x a direction on the
    sphere, in world units: a ray from the interior runs a median 0.4 before
    it meets one, and the slit is in view from about a sixth of the
    interior), every surface Lambert with albedo 0.7, pinhole camera inside
    the room at the image's aspect."""
    f = np.float32
    tris = _box_faces((-2.0, 0.0, 0.0), (2.0, 3.0, 3.0), skip=("x1",))
    # the x = 2 wall below and above the slit (normals toward -x)
    for ya, yb in ((0.0, 2.0), (2.06, 3.0)):
        tris += [(2.0, ya, 0.0), (2.0, ya, 3.0), (2.0, yb, 3.0), (2.0, ya, 0.0), (2.0, yb, 3.0), (2.0, yb, 0.0)]
    # the light chamber (open toward the room)
    tris += _box_faces((2.0, 0.0, 0.0), (2.4, 3.0, 3.0), skip=("x0",))
    room = np.asarray(tris, f)
    c = np.asarray([-1.8, 0.2, 0.3])
    sv, sidx = triangle_soup(n_tris, seed, lo=c, hi=c + np.asarray([3.6, 2.6, 2.5]), edge=0.02)
    shaders = [dict(diffuse_colour=(0.7, 0.7, 0.7), diffuse_strength=1.0, diffuse_roughness=0.0),
               dict(emission_colour=(1.0, 1.0, 1.0), emission_strength=200.0, diffuse_colour=(0.0, 0.0, 0.0),
                    diffuse_strength=1.0, diffuse_roughness=0.0)]
    p0, e1, e2 = (2.35, 0.5, 2.5), (0.0, 2.0, 0.0), (0.0, 0.0, -2.0)
    lv, li = quad_light_mesh(p0, e1, e2)
    meshes = [dict(verts=room, idxp=np.arange(room.shape[0], dtype=np.uint32), shaders=[0]),
              dict(verts=sv, idxp=sidx, shaders=[0]),
              dict(verts=lv, idxp=li, shaders=[1])]
    quads = [dict(p0=p0, e1=e1, e2=e2, shader=1, mesh=2)]
    cam = lookat_camera((-1.2, 1.4, 0.15), (1.0, 1.3, 2.2), (0.0, 1.0, 0.0), 70.0, width / height)
    return dict(meshes=meshes, shaders=shaders, lights=[], quad_lights=quads, env=(0.0, 0.0, 0.0), camera=cam,
                width=width, height=height)


def disk_light_mesh(P, up, lookat, radius: float, segments: int = 20):
    """The emissive fan a DiskLight adds (builtin/light/disk.go:214-258): per
    segment (P, P + R cos(a) B + R sin(a) T, P + R cos(a+da) B + R sin(a+da) T),
    the angle advanced in float32, every vertex normal N; N, T, B from
    Disk.PreRender (disk.go:88-90) in float32."""
    f = np.float32
    P, up, lookat = (np.asarray(a, f) for a in (P, up, lookat))
    N = _norm32(lookat - P)
    T = _norm32(_cross32(N, up))
    B = _cross32(N, T)
    R = f(radius)
    pi = f(3.14159265358)
    dv = f(f(2) * pi) / f(segments)
    ang = f(0)
    verts = []
    for _ in range(segments):
        a1 = f(ang + dv)
        c0, s0 = f(np.cos(np.float64(ang))), f(np.sin(np.float64(ang)))
        c1, s1 = f(np.cos(np.float64(a1))), f(np.sin(np.float64(a1)))
        verts += [P, P + ((R * c0) * B + (R * s0) * T), P + ((R * c1) * B + (R * s1) * T)]
        ang = f(ang + dv)
    v = np.asarray(verts, f)
    return v, np.arange(v.shape[0], dtype=np.uint32), np.tile(N, (v.shape[0], 1)).astype(f)


def small_room_disk(n_tris: int = 4096, seed: int = 1, lens_radius: float = 0.05, light_samples: int = 1) -> dict:
    """The small room lit by one DiskLight (radius 0.2, facing down through
    the ceiling opening, radiance 10) instead of the TriLight panels, seen
    through a thin-lens camera of the given lens radius focused at the
    room's centre."""
    sc = small_room(n_tris, seed=seed, light_samples=light_samples)
    light_shader = sc["lights"][0]["shader"]
    keep = [m for i, m in enumerate(sc["meshes"]) if i not in {l["mesh"] for l in sc["lights"]}]
    P, up, at = (0.0, 1.08, 0.0), (0.0, 0.0, 1.0), (0.0, 0.0, 0.0)
    v, i, n = disk_light_mesh(P, up, at, 0.2)
    keep.append(dict(verts=v, idxp=i, normals=n, shaders=[light_shader]))
    sc["meshes"] = keep
    sc["lights"] = []
    sc["disk_lights"] = [dict(P=P, up=up, lookat=at, radius=0.2, samples=light_samples, shader=light_shader,
                              mesh=len(keep) - 1)]
    cam = lookat_camera((0.0, 0.0, -3.4), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0, 1.0, focal=3.4)
    cam["radius"] = np.float32(lens_radius)
    sc["camera"] = cam
    return sc


def small_room_mirror(n_tris: int = 4096, seed: int = 1, light_samples: int = 1) -> dict:
    """The small room with mirrors (ShaderStd with Spec1Roughness 0): the back
    and side walls pure mirrors (no diffuse weight) facing each other, so
    reflections chain to the deepest level core.Trace evaluates, and half of
    the soup's materials diffuse + mirror (Spec1Strength 0.4, dielectric IOR
    1.5 or a Metal Fresnel)."""
    sc = small_room(n_tris, seed=seed, light_samples=light_samples)
    sh = sc["shaders"]
    for wall in (2, 3, 4):
        sh[wall] = dict(spec1_colour=(0.95, 0.9, 0.85), spec1_strength=1.0, spec1_roughness=0.0,
                        spec1_fresnel="Metal", spec1_fresnel_refl=(0.9, 0.9, 0.9))
    for k, sid in enumerate(range(5, 13)):
        if k % 2 == 0:
            extra = dict(spec1_colour=(1.0, 1.0, 1.0), spec1_strength=0.4, spec1_roughness=0.0, ior=1.5)
            sh[sid] = dict(sh[sid], **extra)
    return sc


def small_room_spheres(n_tris: int = 4096, seed: int = 1, light_samples: int = 1) -> dict:
    """The small room lit by a SphereLight (radius 0.12 hanging below the
    ceiling, radiance 10) besides the TriLight panels, with three analytic
    sphere geoms (builtin/geom/sphere) on the floor: Lambert, diffuse + GGX,
    and a mirror."""
    sc = small_room(n_tris, seed=seed, light_samples=light_samples)
    sh = sc["shaders"]
    light_shader = sc["lights"][0]["shader"]
    base = len(sh)
    sh += [dict(diffuse_colour=(0.8, 0.3, 0.3), diffuse_strength=1.0, diffuse_roughness=0.0),
           dict(diffuse_colour=(0.3, 0.8, 0.3), diffuse_strength=0.7, diffuse_roughness=0.0,
                spec1_colour=(1.0, 1.0, 1.0), spec1_strength=0.3, spec1_roughness=0.4, ior=1.5),
           dict(spec1_colour=(0.9, 0.9, 0.9), spec1_strength=1.0, spec1_roughness=0.0, ior=1.5)]
    for k, (x, z) in enumerate(((-0.5, 0.3), (0.0, 0.5), (0.5, 0.2))):
        sc["meshes"].append(dict(sphere=(x, -0.75, z, 0.25), shaders=[base + k]))
    sc["meshes"].append(dict(sphere=(0.0, 0.6, 0.0, 0.12), shaders=[light_shader]))
    sc["sphere_lights"] = [dict(P=(0.0, 0.6, 0.0), radius=0.12, samples=light_samples, shader=light_shader,
                                mesh=len(sc["meshes"]) - 1)]
    return sc


def small_room_motion(n_tris: int = 4096, seed: int = 1, motion_mode: int = 0, velocity: float = 0.08,
                      normals: bool = False) -> dict:
    """The small room with its soup moving: two motion keys (key 1 = key 0 +
    a per-triangle velocity in a ball of the given radius), sampled over the
    shutter by each camera ray's VdC time; motion_mode 0 reproduces
    TraceMotionElems' leaf indexing, 1 the face the leaf boxes bound.
    normals: per-key corner normals for the soup (motion_normals [2, 3n, 3]:
    each key's face normal tilted by a seeded random vector of length 0.5 per
    corner, unit length)."""
    sc = small_room(n_tris, seed=seed)
    soup = sc["meshes"][1]
    v0 = soup["verts"].reshape(n_tris, 3, 3).astype(np.float64)
    d = unit_sphere(seed, n_tris, 40) * (velocity * np.cbrt(uniform(seed, n_tris, 42)))[:, None]
    v1 = (v0 + d[:, None, :]).astype(np.float32).reshape(-1, 3)
    soup["verts"] = np.concatenate([soup["verts"], v1], axis=0)
    soup["keys"] = 2
    soup["motion_mode"] = motion_mode
    if normals:
        keys = []
        for k, vk in enumerate((v0, v1.reshape(n_tris, 3, 3).astype(np.float64))):
            fn = np.cross(vk[:, 1] - vk[:, 0], vk[:, 2] - vk[:, 0])
            fn /= np.maximum(np.linalg.norm(fn, axis=1, keepdims=True), 1e-30)
            c = np.repeat(fn, 3, axis=0) + 0.5 * unit_sphere(seed, 3 * n_tris, 50 + k)
            keys.append(c / np.maximum(np.linalg.norm(c, axis=1, keepdims=True), 1e-30))
        soup["motion_normals"] = np.stack(keys).astype(np.float32)
    return sc


def xf_matrix(angle, axis, scale, translate) -> np.ndarray:
    """Column-major 4x4 (math.Matrix4 order) of x -> translate + R(angle,
    axis) diag(scale) x, as float32."""
    axis = np.asarray(axis, np.float64) / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K
    A = np.eye(4)
    A[:3, :3] = R @ np.diag(scale)
    A[:3, 3] = translate
    return A.T.reshape(16).astype(np.float32)


def _box_of(verts, keys16, margin=0.02):
    """A box around the vertices under every key (for BMin/BMax)."""
    v = np.asarray(verts, np.float64).reshape(-1, 3)
    lo, hi = np.full(3, np.inf), np.full(3, -np.inf)
    for k in np.asarray(keys16, np.float64).reshape(-1, 16):
        A = k.reshape(4, 4).T
        w = v @ A[:3, :3].T + A[:3, 3]
        lo, hi = np.minimum(lo, w.min(0)), np.maximum(hi, w.max(0))
    # keys blend rotations on arcs between the keys: grow the box by its half size
    pad = 0.5 * (hi - lo) + margin
    return (lo - pad).astype(np.float32), (hi + pad).astype(np.float32)


def small_room_groups(n_tris: int = 4096, seed: int = 1, camera_keys: bool = True, debug: bool = True) -> dict:
    """The small room with the node types that reach geometry through
    transforms: an object (a 600-triangle soup in a 0.3 cube about the
    origin, itself placed in the room), two GeomInstances of it (one key; two
    keys moving and turning over the shutter), an instance of an analytic
    sphere, a Proc of two meshes (one with its own PolyMesh transform) under
    two transform keys, a mesh with two PolyMesh transform keys, a
    DebugShader on the instanced object and the back wall (debug; else their
    ShaderStd shaders), and (camera_keys) two camera motion keys."""
    sc = small_room(n_tris, seed=seed)
    M = sc["meshes"]
    shaders = sc["shaders"]
    debug_id = len(shaders)
    shaders.append(dict(debug=True, diffuse_colour=(0.9, 0.2, 0.6)))
    ov, oi = triangle_soup(600, seed + 90, lo=-0.15, hi=0.15, edge=0.04)
    obj = dict(verts=ov, idxp=oi, shaders=[5, 6], face_shader=(np.arange(600) % 2).astype(np.uint8),
               transform=xf_matrix(0.0, (0, 1, 0), (1, 1, 1), (-0.5, -0.55, 0.3)))
    M.append(obj)
    i_obj = len(M) - 1
    ow = ov.reshape(-1, 3) + np.float32([-0.5, -0.55, 0.3])  # the object under its own transform
    k1 = [xf_matrix(0.7, (0, 1, 0), (1.3, 0.8, 1.0), (0.45, 0.2, -0.2))]
    lo, hi = _box_of(ow, k1)
    M.append(dict(instance=i_obj, keys=k1, bmin=lo, bmax=hi, shaders=[]))
    k2 = [xf_matrix(0.2, (1, 1, 0), (1, 1, 1), (0.4, 0.85, -0.4)),
          xf_matrix(0.9, (1, 1, 0), (1.2, 1.2, 1.2), (0.52, 0.92, -0.35))]
    lo, hi = _box_of(ow, k2)
    M.append(dict(instance=i_obj, keys=k2, bmin=lo, bmax=hi, shaders=[]))
    # (off the origin: two geoms with one box centroid, here the room's, make
    # the reference's top-level split recurse forever, qbvh/build.go:34-43)
    M.append(dict(sphere=(0.03, 0.02, -0.01, 0.12), shaders=[7]))
    i_sph = len(M) - 1
    k3 = [xf_matrix(0.0, (0, 0, 1), (1.0, 1.5, 1.0), (-0.48, 0.23, -0.44))]
    lo, hi = _box_of(np.array([[-0.09, -0.1, -0.13], [0.15, 0.14, 0.11]]), k3, margin=0.2)
    M.append(dict(instance=i_sph, keys=k3, bmin=lo, bmax=hi, shaders=[]))
    # a Proc's children: meshes made for it (they join no scene themselves)
    av, ai = triangle_soup(400, seed + 91, lo=-0.12, hi=0.12, edge=0.03)
    bv, bi = triangle_soup(300, seed + 92, lo=-0.1, hi=0.1, edge=0.03)
    M.append(dict(verts=av, idxp=ai, shaders=[8]))
    ca = len(M) - 1
    M.append(dict(verts=bv, idxp=bi, shaders=[9], transform=xf_matrix(0.4, (0, 0, 1), (1, 1, 1), (0.1, 0.05, 0.0))))
    cb = len(M) - 1
    k4 = [xf_matrix(0.0, (0, 1, 0), (1, 1, 1), (0.5, 0.3, 0.4)), xf_matrix(0.5, (0, 1, 0), (1, 1, 1), (0.45, 0.3, 0.5))]
    lo, hi = _box_of(np.concatenate([av, bv + 0.12]), k4, margin=0.1)
    M.append(dict(proc=[ca, cb], keys=k4, bmin=lo, bmax=hi, shaders=[]))
    # a mesh with two PolyMesh transform keys
    tv, ti = triangle_soup(500, seed + 93, lo=-0.12, hi=0.12, edge=0.03)
    M.append(dict(verts=tv, idxp=ti, shaders=[10, 11], face_shader=(np.arange(500) % 2).astype(np.uint8),
                  transform_keys=[xf_matrix(0.0, (1, 0, 0), (1, 1, 1), (-0.1, -0.3, -0.6)),
                                  xf_matrix(0.8, (1, 0, 0), (1.1, 1.1, 1.1), (0.05, -0.25, -0.55))]))
    if debug:
        obj["shaders"] = [debug_id, 6]
        M[0]["shaders"] = [0, 1, debug_id, 3, 4]  # the back wall too
    if camera_keys:
        cam = sc["camera"]
        m0 = np.asarray(cam["m"], np.float32)
        m1 = m0.copy()
        m1[12:15] += np.float32([0.08, 0.03, 0.0])
        cam["keys"] = np.stack([m0, m1])
    return sc


# ------------------------------------------------------------ .vnf files ---
def _vnf_num(x) -> str:
    """A float32 value as the decimal of its exact double (read back through
    float64, as the reference's lexer does, it gives the same float32)."""
    return repr(float(np.float32(x)))


def _light_mesh_ids(scene: dict) -> set:
    ids = set()
    for k in ("lights", "disk_lights", "sphere_lights", "quad_lights"):
        ids |= {int(l["mesh"]) for l in scene.get(k, [])}
    return ids


def _mat_rows(keys) -> str:
    """Matrices (column-major 16 each) as the parser reads them: row by row
    (the reader transposes)."""
    a = np.asarray(keys, np.float32).reshape(-1, 16)
    return " ".join(_vnf_num(x) for k in a for x in k.reshape(4, 4).T.ravel())


def _geom_node(gi: int, m: dict) -> str:
    if "sphere" in m:
        c = m["sphere"]
        return (f'Sphere {{\n  Name "geom{gi}"\n  P {_vnf_num(c[0])} {_vnf_num(c[1])} {_vnf_num(c[2])}\n'
                f'  Radius {_vnf_num(c[3])}\n  Shader "sh{m["shaders"][0]}"\n}}')
    keys = int(m.get("keys", 1))
    v = np.asarray(m["verts"], np.float32).reshape(-1, 3)
    per = v.shape[0] // keys
    idx = np.asarray(m["idxp"], np.uint32)
    lines = [f'PolyMesh {{\n  Name "geom{gi}"',
             f"  Verts {keys} {per} point " + " ".join(_vnf_num(x) for x in v.ravel()),
             f"  FaceIdx {idx.size} int " + " ".join(str(int(x)) for x in idx),
             f"  Shader {len(m['shaders'])} string " + " ".join(f'"sh{s}"' for s in m["shaders"])]
    if m.get("face_shader") is not None:
        fs = np.asarray(m["face_shader"], np.uint8)
        lines.append(f"  ShaderIdx {fs.size} int " + " ".join(str(int(x)) for x in fs))
    if m.get("motion_normals") is not None:  # as many keys as the vertices
        nr = np.asarray(m["motion_normals"], np.float32)
        lines.append(f"  Normals {nr.shape[0]} {nr.shape[1]} vec3 " + " ".join(_vnf_num(x) for x in nr.ravel()))
    elif m.get("normals") is not None:
        nr = np.asarray(m["normals"], np.float32).reshape(-1, 3)
        lines.append(f"  Normals 1 {nr.shape[0]} vec3 " + " ".join(_vnf_num(x) for x in nr.ravel()))
    if m.get("transform_keys") is not None:
        k = np.asarray(m["transform_keys"], np.float32).reshape(-1, 16)
        lines.append(f"  Transform {k.shape[0]} matrix " + _mat_rows(k))
    elif m.get("transform") is not None:
        lines.append("  Transform 1 matrix " + _mat_rows(m["transform"]))
    return "\n".join(lines) + "\n}"


def to_vnf(scene: dict, width: int, height: int, max_iter: int = 16, extra_files: dict | None = None) -> str:
    """The scene as a .vnf file the reference's parser (nodes/parser.go) and
    vmr_load_vnf read: ShaderStd (or DebugShader) nodes "sh<i>", a PolyMesh,
    Sphere, GeomInstance or Proc node per geom that is neither a light's own
    mesh nor a Proc's child, the lights (which create their meshes when
    loaded), a matrix Camera "camera" with the scene camera's LocalToWorld
    keys, Fov and Focal, Globals, and the pixel filter if any.  A Proc's
    children go to a file of their own that its Data names (Handler "vnf"):
    extra_files receives {name: text} for those.  The environment light has
    no node in the reference and is not written."""
    out = []
    for i, d in enumerate(scene["shaders"]):
        if d.get("debug"):
            out.append(f'DebugShader {{\n  Name "sh{i}"\n  Colour rgb ' +
                       " ".join(_vnf_num(x) for x in d["diffuse_colour"]) + "\n}")
            continue
        out.append(f'ShaderStd {{\n  Name "sh{i}"')
        names = {"emission_colour": "EmissionColour", "emission_strength": "EmissionStrength",
                 "diffuse_colour": "DiffuseColour", "diffuse_strength": "DiffuseStrength",
                 "diffuse_roughness": "DiffuseRoughness", "spec1_colour": "Spec1Colour",
                 "spec1_strength": "Spec1Strength", "spec1_roughness": "Spec1Roughness",
                 "spec1_fresnel_refl": "Spec1FresnelRefl", "spec1_fresnel_edge": "Spec1FresnelEdge", "ior": "IOR"}
        for k, node in names.items():
            if k in d:
                v = d[k]
                if np.ndim(v) == 0:
                    out.append(f"  {node} float {_vnf_num(v)}")
                else:
                    out.append(f"  {node} rgb " + " ".join(_vnf_num(x) for x in v))
        if "spec1_fresnel" in d:
            out.append(f'  Spec1FresnelModel "{d["spec1_fresnel"]}"')
        out.append("}")
    lights = _light_mesh_ids(scene)
    children = {c for m in scene["meshes"] if "proc" in m for c in m["proc"]}
    pt = lambda a: "1 1 point " + " ".join(_vnf_num(x) for x in a)  # noqa: E731
    for gi, m in enumerate(scene["meshes"]):
        if gi in lights or gi in children:
            continue
        if "instance" in m:
            k = np.asarray(m["keys"], np.float32).reshape(-1, 16)
            out.append(f'GeomInstance {{\n  Name "geom{gi}"\n  Geom "geom{m["instance"]}"\n  BMin {pt(m["bmin"])}\n'
                       f'  BMax {pt(m["bmax"])}\n  Transform {k.shape[0]} matrix {_mat_rows(k)}\n}}')
        elif "proc" in m:
            name = f"proc{gi}.vnf"
            if extra_files is not None:
                extra_files[name] = "\n".join(_geom_node(c, scene["meshes"][c]) for c in m["proc"]) + "\n"
            lines = [f'Proc {{\n  Name "geom{gi}"\n  Handler "vnf"\n  Data "{name}"',
                     f"  BMin {pt(m['bmin'])}\n  BMax {pt(m['bmax'])}"]
            if m.get("keys") is not None:
                k = np.asarray(m["keys"], np.float32).reshape(-1, 16)
                lines.append(f"  Transform {k.shape[0]} matrix {_mat_rows(k)}")
            out.append("\n".join(lines) + "\n}")
        else:
            out.append(_geom_node(gi, m))
    vec = lambda a: " ".join(_vnf_num(x) for x in a)  # noqa: E731
    for i, l in enumerate(scene.get("lights", [])):
        out.append(f'TriLight {{\n  Name "tri{i}"\n  P0 {vec(l["p0"])}\n  P1 {vec(l["p1"])}\n  P2 {vec(l["p2"])}\n'
                   f'  Shader "sh{l["shader"]}"\n  Samples {int(l.get("samples", 1))}\n}}')
    for i, l in enumerate(scene.get("disk_lights", [])):
        out.append(f'DiskLight {{\n  Name "disk{i}"\n  P {vec(l["P"])}\n  Up {vec(l["up"])}\n'
                   f'  LookAt {vec(l["lookat"])}\n  Radius {_vnf_num(l["radius"])}\n  Shader "sh{l["shader"]}"\n'
                   f'  Samples {int(l.get("samples", 1))}\n}}')
    for i, l in enumerate(scene.get("sphere_lights", [])):
        out.append(f'SphereLight {{\n  Name "sphere{i}"\n  P {vec(l["P"])}\n  Radius {_vnf_num(l["radius"])}\n'
                   f'  Shader "sh{l["shader"]}"\n  Samples {int(l.get("samples", 1))}\n}}')
    for i, l in enumerate(scene.get("quad_lights", [])):
        out.append(f'QuadLight {{\n  Name "quad{i}"\n  P {vec(l["p0"])}\n  U {vec(l["e1"])}\n  V {vec(l["e2"])}\n'
                   f'  Shader "sh{l["shader"]}"\n}}')
    c = scene["camera"]
    ck = np.asarray(c["keys"] if c.get("keys") is not None else c["m"], np.float32).reshape(-1, 16)
    out.append('Camera {\n  Name "camera"\n  Type "matrix"\n  From 1 1 point 0 0 0\n  To 1 1 point 0 0 -1\n'
               '  Roll 1 1 float 0\n  Up 0 1 0\n'
               f'  Fov {_vnf_num(c.get("fov", 90.0))}\n  Focal {_vnf_num(c["focal"])}\n'
               f'  Aspect {_vnf_num(c["aspect"])}\n  Radius {_vnf_num(c["radius"])}\n'
               f"  LocalToWorld {ck.shape[0]} matrix {_mat_rows(ck)}\n}}")
    out.append(f"Globals {{\n  XRes {int(width)}\n  YRes {int(height)}\n  MaxIter {int(max_iter)}\n}}")
    pf = scene.get("pixel_filter")
    if pf:
        if int(pf["kind"]) == 1:
            out.append(f'GaussianFilter {{\n  Name "filter"\n  Width {_vnf_num(pf.get("width", 2.0))}\n'
                       f'  Res {int(pf.get("res", 17))}\n}}')
        else:
            out.append(f'AiryFilter {{\n  Name "filter"\n  Width {_vnf_num(pf.get("width", 6.0))}\n'
                       f'  Res {int(pf.get("res", 49))}\n  Peak {_vnf_num(pf.get("peak", 4.0))}\n}}')
    return "# written by vermeer_gb300.scenes.to_vnf\n" + "\n".join(out) + "\n"


def vnf_order(scene: dict) -> dict:
    """The scene as vmr_load_vnf builds it from to_vnf's file: the geoms that
    are not lights' meshes in their order, then the lights' meshes in the
    order TriLights, DiskLights, SphereLights, QuadLights (each quad as the
    reference's 4-vertex polygon with its normal, quad.go:174-207), the
    light tables pointing at the new positions, and no environment."""
    lights = _light_mesh_ids(scene)
    order = [g for g in range(len(scene["meshes"])) if g not in lights]
    meshes = [scene["meshes"][g] for g in order]
    out = dict(scene, env=(0.0, 0.0, 0.0))
    for key in ("lights", "disk_lights", "sphere_lights", "quad_lights"):
        new = []
        for l in scene.get(key, []):
            m = scene["meshes"][int(l["mesh"])]
            if key == "quad_lights":
                f = np.float32
                P, U, V = (np.asarray(l[k], f) for k in ("p0", "e1", "e2"))
                c = np.stack([P, (P + U).astype(f), ((P + U).astype(f) + V).astype(f), (P + V).astype(f)]).astype(f)
                N = _norm32(_cross32(U, V))
                m = dict(verts=c, idxp=np.array([0, 1, 2, 0, 2, 3], np.uint32), shaders=[int(l["shader"])],
                         normals=np.tile(N, (4, 1)).astype(f))
            new.append(dict(l, mesh=len(meshes)))
            meshes.append(m)
        out[key] = new
    out["meshes"] = meshes
    return out


def batched_jobs(n_jobs: int = 64, seed: int = 4, width: int = 256, height: int = 256,
                 lo: int = 1000, hi: int = 200_000) -> dict:
    """The batched-jobs configuration: n_jobs triangle soups (the raw-traversal
    soup's construction: centroids in the unit cube, 0.005 edges) with sizes
    log-uniform in [lo, hi] (seed), every other one with two-key linear
    motion (per-triangle velocity uniform in a 0.05 ball, shutter [0, 1]);
    each job renders its soup alone through a pinhole looking into the cube,
    Lambert albedo 0.7 under a constant white environment (the configuration
    names no material or light).  Returns dict(meshes, shaders, env, cameras,
    width, height): meshes[j] is job j's mesh, cameras[j] its camera."""
    sizes = np.exp(np.log(lo) + (np.log(hi) - np.log(lo)) * uniform(seed, n_jobs, 0)).astype(int)
    meshes = []
    for j, nt in enumerate(sizes):
        if j % 2 == 1:
            v, ip = motion_soup(int(nt), 400 + j, velocity=0.05)
            meshes.append(dict(verts=v, idxp=ip, keys=2, motion_mode=1, shaders=[0]))
        else:
            v, ip = triangle_soup(int(nt), 400 + j)
            meshes.append(dict(verts=v, idxp=ip, shaders=[0]))
    cam = lookat_camera((0.5, 0.5, -1.2), (0.5, 0.5, 0.5), (0.0, 1.0, 0.0), 40.0, width / height)
    return dict(meshes=meshes, shaders=[dict(diffuse_colour=(0.7, 0.7, 0.7), diffuse_strength=1.0,
                                             diffuse_roughness=0.0)],
                env=(1.0, 1.0, 1.0), cameras=[cam] * n_jobs, width=width, height=height, sizes=sizes)
