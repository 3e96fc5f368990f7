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
