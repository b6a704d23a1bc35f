"""Seeded synthetic workloads for the ray-tracing hot path.

The reference measures on no public dataset; its real scenes (sponza etc.) are
not shipped.  These generators define the workloads instead:

* ``random_triangles`` / ``sphere_rays``: 65,536 random small triangles and
  1,048,576 rays aimed into the unit cube from a radius-2 sphere.
* ``terrain_boxes``: a 512x512 value-noise heightfield over [0,100]^2
  (524,288 triangles) plus 200 boxes standing on it (2,400 triangles).
* ``pinhole_rays``: a 1920x1080 pinhole primary pass with a 60 degree
  vertical field of view, ray direction formed like the reference's ray-gen
  shader (data/shader/pathtracer/rayGen.csh:44-48).
* ``batched_scenes``: 64 independent random-triangle scenes with log-uniform
  sizes and ray batches.

Every value is produced with float32 arithmetic that rounds the same on any
IEEE host (no transcendental functions, explicit evaluation order), so x86-64
and aarch64 hosts generate bit-identical inputs from the same seed.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32
DEFAULT_SEED = 0xA71A5


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def _normalize(v: np.ndarray) -> np.ndarray:
    """float32 normalisation v * (1 / sqrt((x*x + y*y) + z*z))."""
    v = v.astype(F32, copy=False)
    d = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
    inv = F32(1.0) / np.sqrt(d, dtype=F32)
    return (v * inv[:, None]).astype(F32)


def _unit_vectors(rng: np.random.Generator, n: int) -> np.ndarray:
    """Directions uniform on the sphere by rejection from the cube."""
    out = np.empty((n, 3), np.float64)
    filled = 0
    while filled < n:
        c = rng.random((max(2 * (n - filled), 1024), 3)) * 2.0 - 1.0
        r2 = (c[:, 0] * c[:, 0] + c[:, 1] * c[:, 1]) + c[:, 2] * c[:, 2]
        keep = c[(r2 <= 1.0) & (r2 > 1e-6)]
        take = min(len(keep), n - filled)
        out[filled:filled + take] = keep[:take]
        filled += take
    r = np.sqrt((out[:, 0] * out[:, 0] + out[:, 1] * out[:, 1]) + out[:, 2] * out[:, 2])
    return (out / r[:, None]).astype(F32)


# --------------------------------------------------------------------------
# Random triangles (the plain ray-cast workload)
# --------------------------------------------------------------------------

def random_triangles(n_tris: int = 65536, seed: int = DEFAULT_SEED) -> np.ndarray:
    """(n, 3, 3) float32: centroid ~ U[0,1]^3, each vertex = centroid + U[-0.01,0.01]^3."""
    rng = _rng(seed)
    centroid = rng.random((n_tris, 1, 3)).astype(F32)
    offs = (rng.random((n_tris, 3, 3)) * 0.02 - 0.01).astype(F32)
    return (centroid + offs).astype(F32)


def sphere_rays(n_rays: int = 1 << 20, seed: int = DEFAULT_SEED + 1,
                radius: float = 2.0, center=(0.5, 0.5, 0.5)):
    """Origins uniform on a sphere of `radius` around `center`, each aimed at
    its own uniform point in [0,1]^3.  Returns (origins, dirs), float32 (n,3)."""
    rng = _rng(seed)
    n_hat = _unit_vectors(rng, n_rays)
    c = np.asarray(center, F32)
    origins = (c[None, :] + F32(radius) * n_hat).astype(F32)
    target = rng.random((n_rays, 3)).astype(F32)
    dirs = _normalize(target - origins)
    return origins, dirs


# --------------------------------------------------------------------------
# Terrain + boxes
# --------------------------------------------------------------------------

def _hash32(a: np.ndarray) -> np.ndarray:
    """Integer avalanche hash on uint32 (xorshift-multiply)."""
    x = a.astype(np.uint32)
    x ^= x >> np.uint32(16)
    x = (x * np.uint32(0x7FEB352D)).astype(np.uint32)
    x ^= x >> np.uint32(15)
    x = (x * np.uint32(0x846CA68B)).astype(np.uint32)
    x ^= x >> np.uint32(16)
    return x


def _lattice(seed: int, octave: int, ix: np.ndarray, iz: np.ndarray) -> np.ndarray:
    """Lattice value in [0,1) at integer point (ix, iz) of one octave."""
    with np.errstate(over="ignore"):
        k = (ix.astype(np.uint32) * np.uint32(73856093)) ^ (iz.astype(np.uint32) * np.uint32(19349663))
        k = k ^ np.uint32((seed * 2654435761 + octave * 40503) & 0xFFFFFFFF)
        h = _hash32(k)
    return ((h >> np.uint32(8)).astype(F32) * F32(1.0 / 16777216.0)).astype(F32)


def value_noise(seed: int, octave: int, x: np.ndarray, z: np.ndarray, freq: float) -> np.ndarray:
    """Smoothstep-interpolated value noise, `freq` lattice cells per 100 units."""
    fx = (x.astype(F32) * F32(freq / 100.0)).astype(F32)
    fz = (z.astype(F32) * F32(freq / 100.0)).astype(F32)
    ix = np.floor(fx)
    iz = np.floor(fz)
    tx = (fx - ix).astype(F32)
    tz = (fz - iz).astype(F32)
    sx = (tx * tx * (F32(3.0) - F32(2.0) * tx)).astype(F32)
    sz = (tz * tz * (F32(3.0) - F32(2.0) * tz)).astype(F32)
    ix = ix.astype(np.int64)
    iz = iz.astype(np.int64)
    v00 = _lattice(seed, octave, ix, iz)
    v10 = _lattice(seed, octave, ix + 1, iz)
    v01 = _lattice(seed, octave, ix, iz + 1)
    v11 = _lattice(seed, octave, ix + 1, iz + 1)
    a = v00 + sx * (v10 - v00)
    b = v01 + sx * (v11 - v01)
    return (a + sz * (b - a)).astype(F32)


def terrain_height(seed: int, x: np.ndarray, z: np.ndarray,
                   octaves: int = 4, amplitude: float = 10.0, base_freq: float = 4.0) -> np.ndarray:
    """Sum over octaves o of amplitude * 2^-o * noise(freq * 2^o)."""
    h = np.zeros(np.broadcast(x, z).shape, F32)
    for o in range(octaves):
        amp = F32(amplitude * (0.5 ** o))
        h = (h + amp * value_noise(seed, o, x, z, base_freq * (2 ** o))).astype(F32)
    return h


def _box_triangles(lo: np.ndarray, hi: np.ndarray) -> np.ndarray:
    """12 triangles of an axis-aligned box, outward winding. (12, 3, 3)."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    c = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], F32)
    faces = [(0, 3, 2), (0, 2, 1),   # -z
             (4, 5, 6), (4, 6, 7),   # +z
             (0, 4, 7), (0, 7, 3),   # -x
             (1, 2, 6), (1, 6, 5),   # +x
             (0, 1, 5), (0, 5, 4),   # -y
             (3, 7, 6), (3, 6, 2)]   # +y
    return c[np.array(faces)]


def terrain_boxes(seed: int = DEFAULT_SEED, grid: int = 512, extent: float = 100.0,
                  n_boxes: int = 200):
    """Heightfield + boxes.  Returns (tris (n,3,3) float32, object_id (n,) int32).

    object_id is 0 for the terrain and 1 + b for box b (used for materials).
    """
    coords = (np.arange(grid + 1, dtype=F32) * F32(extent / grid)).astype(F32)
    X, Z = np.meshgrid(coords, coords, indexing="ij")
    H = terrain_height(seed, X, Z)
    P = np.stack([X, H, Z], axis=-1).astype(F32)            # (g+1, g+1, 3)
    p00 = P[:-1, :-1].reshape(-1, 3)
    p10 = P[1:, :-1].reshape(-1, 3)
    p01 = P[:-1, 1:].reshape(-1, 3)
    p11 = P[1:, 1:].reshape(-1, 3)
    # two triangles per cell, wound so that the face normal points up (+y)
    t0 = np.stack([p00, p11, p10], axis=1)
    t1 = np.stack([p00, p01, p11], axis=1)
    terrain = np.stack([t0, t1], axis=1).reshape(-1, 3, 3)

    rng = _rng(seed + 7)
    centers = (rng.random((n_boxes, 2)) * (extent * 0.9) + extent * 0.05).astype(F32)
    sides = (rng.random((n_boxes, 3)) * 4.0 + 1.0).astype(F32)
    ground = terrain_height(seed, centers[:, 0], centers[:, 1])
    boxes = []
    for b in range(n_boxes):
        lo = np.array([centers[b, 0] - sides[b, 0] * F32(0.5), ground[b] - F32(0.5),
                       centers[b, 1] - sides[b, 2] * F32(0.5)], F32)
        hi = np.array([centers[b, 0] + sides[b, 0] * F32(0.5), ground[b] - F32(0.5) + sides[b, 1],
                       centers[b, 1] + sides[b, 2] * F32(0.5)], F32)
        boxes.append(_box_triangles(lo, hi))
    boxes = np.concatenate(boxes, axis=0)
    tris = np.concatenate([terrain, boxes], axis=0).astype(F32)
    obj = np.concatenate([np.zeros(len(terrain), np.int32),
                          1 + np.repeat(np.arange(n_boxes, dtype=np.int32), 12)])
    return np.ascontiguousarray(tris), obj


# --------------------------------------------------------------------------
# Camera
# --------------------------------------------------------------------------

def pinhole_camera(width: int = 1920, height: int = 1080, fov_deg: float = 60.0,
                   eye=(50.0, 45.0, -22.0), target=(50.0, 0.0, 48.0), up=(0.0, 1.0, 0.0)):
    """Frustum description in the reference's ray-gen form (PathTracingRenderer.cpp:157-160):
    the image-plane corner `origin` (top-left) and the `right` / `bottom` spans at
    unit distance, plus the camera location.  Returns a dict of float32 3-vectors."""
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, np.asarray(up, np.float64))
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    half_h = np.tan(np.radians(fov_deg) * 0.5)
    half_w = half_h * width / height
    corner = eye + fwd - right * half_w + upv * half_h
    return {
        "location": eye.astype(F32),
        "origin": corner.astype(F32),
        "right": (right * 2.0 * half_w).astype(F32),
        "bottom": (-upv * 2.0 * half_h).astype(F32),
        "width": width, "height": height,
    }


def pinhole_rays(cam: dict, jitter=(0.5, 0.5)):
    """Primary rays, pixel-major order: dir = normalize(origin + right*u + bottom*v - location)
    with (u, v) = (pixel + jitter) / resolution.  Returns (origins, dirs) float32 (n,3)."""
    w, h = cam["width"], cam["height"]
    px = np.arange(w, dtype=F32)
    py = np.arange(h, dtype=F32)
    u = ((px + F32(jitter[0])) / F32(w)).astype(F32)
    v = ((py + F32(jitter[1])) / F32(h)).astype(F32)
    U, V = np.meshgrid(u, v, indexing="xy")
    U = U.reshape(-1, 1)
    V = V.reshape(-1, 1)
    p = (cam["origin"][None, :] + cam["right"][None, :] * U) + cam["bottom"][None, :] * V
    d = _normalize((p - cam["location"][None, :]).astype(F32))
    o = np.broadcast_to(cam["location"], d.shape).astype(F32)
    return np.ascontiguousarray(o), d


# --------------------------------------------------------------------------
# Batched multi-scene workload
# --------------------------------------------------------------------------

def batched_scenes(n_scenes: int = 64, seed: int = DEFAULT_SEED + 100,
                   tri_range=(1000, 500000), ray_range=(4096, 1 << 20)):
    """Scene and batch sizes, log-uniform.  Returns a list of dicts with
    'n_tris', 'n_rays', 'any' (bool: any-hit batch), 'seed'.  Closest/any batches
    alternate, so the mix is equal."""
    import math
    rng = _rng(seed)
    u = rng.random((n_scenes, 2))
    out = []

    def logu(lo, hi, x):
        # sizes rounded to a multiple of 32, so a last-bit difference between
        # two hosts' exp/log cannot change them
        v = math.exp(math.log(lo) + x * (math.log(hi) - math.log(lo)))
        return max(lo, min(hi, int(round(v / 32.0)) * 32))

    for i in range(n_scenes):
        out.append({"n_tris": logu(tri_range[0], tri_range[1], float(u[i, 0])),
                    "n_rays": logu(ray_range[0], ray_range[1], float(u[i, 1])),
                    "any": bool(i % 2), "seed": int(seed + 1000 + i)})
    return out


# --------------------------------------------------------------------------
# Ray packing in the reference's 48-byte PackedRay layout
# --------------------------------------------------------------------------

def pack_rays(origins: np.ndarray, dirs: np.ndarray, ids: np.ndarray | None = None) -> np.ndarray:
    """(n, 12) float32 view of PackedRay {vec4 origin (w = ID bits); vec4 direction; vec4 hit}
    (data/shader/raytracer/structures.hsh:9-13)."""
    n = len(origins)
    out = np.zeros((n, 12), F32)
    out[:, 0:3] = origins
    out[:, 4:7] = dirs
    if ids is None:
        ids = np.arange(n, dtype=np.int32)
    out[:, 3] = np.asarray(ids, np.int32).view(F32)
    return out


def rays8(origins: np.ndarray, dirs: np.ndarray, tmin: float, tmax: float) -> np.ndarray:
    """(n, 8) float32 rows (origin, dir, tmin, tmax) for the host query oracles."""
    n = len(origins)
    out = np.empty((n, 8), F32)
    out[:, 0:3] = origins
    out[:, 3:6] = dirs
    out[:, 6] = tmin
    out[:, 7] = tmax
    return out
