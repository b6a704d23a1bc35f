"""Rays whose two nearest hits lie within float rounding of each other, on a
small terrain + boxes scene (64 x 64 grid, 20 boxes standing 0.5 deep in the
ground): rays aimed at shared edges and vertices of the terrain grid, at
edges of the box faces, and at the contact lines where a box wall meets the
terrain.  Shared by the oracle's and the GPU's near-tie tests."""
import numpy as np

from atlas_rt import scenes

import pyoracle


def near_tie_scene():
    return scenes.terrain_boxes(grid=64, n_boxes=20)


def _down_dirs(rng, n, spread=0.5):
    d = np.stack([rng.uniform(-spread, spread, n), -np.ones(n), rng.uniform(-spread, spread, n)], 1)
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def near_tie_rays(tris, obj, n_edge=40000, n_vertex=10000, n_box_edge=25000, n_contact=25000, seed=11):
    """(n, 8) float32 rays (origin, direction, tmin 1e-4, tmax 1e4), each 30
    units before its target point, plus a label per ray (0 grid edge,
    1 grid vertex, 2 box edge, 3 contact line)."""
    rng = np.random.default_rng(seed)
    terrain = np.nonzero(obj == 0)[0]
    boxes = np.nonzero(obj > 0)[0]
    tgt, dirs, lab = [], [], []
    # points on terrain triangle edges (shared with the neighbouring triangle)
    pick = terrain[rng.integers(0, len(terrain), n_edge)]
    e = rng.integers(0, 3, n_edge)
    a = tris[pick, e].astype(np.float64)
    b = tris[pick, (e + 1) % 3].astype(np.float64)
    f = rng.uniform(0.02, 0.98, n_edge)[:, None]
    tgt.append(a + f * (b - a)); dirs.append(_down_dirs(rng, n_edge)); lab.append(np.zeros(n_edge, int))
    # terrain vertices
    pick = terrain[rng.integers(0, len(terrain), n_vertex)]
    tgt.append(tris[pick, rng.integers(0, 3, n_vertex)].astype(np.float64))
    dirs.append(_down_dirs(rng, n_vertex)); lab.append(np.ones(n_vertex, int))
    # box triangle edges (face diagonals and box edges), from any side
    pick = boxes[rng.integers(0, len(boxes), n_box_edge)]
    e = rng.integers(0, 3, n_box_edge)
    a = tris[pick, e].astype(np.float64)
    b = tris[pick, (e + 1) % 3].astype(np.float64)
    f = rng.uniform(0.02, 0.98, n_box_edge)[:, None]
    d = rng.normal(size=(n_box_edge, 3))
    d[:, 1] = -np.abs(d[:, 1])
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tgt.append(a + f * (b - a)); dirs.append(d); lab.append(np.full(n_box_edge, 2))
    # contact lines: points of the box walls at the terrain's height there,
    # approached from outside the box and from above
    nb = int(obj.max())
    per = n_contact // (4 * nb) + 1
    pts, dd = [], []
    for k in range(1, nb + 1):
        bt = tris[obj == k].reshape(-1, 3)
        lo, hi = bt.min(0).astype(np.float64), bt.max(0).astype(np.float64)
        for face in range(4):
            s = rng.uniform(0.02, 0.98, per)
            if face < 2:      # walls x = lo.x / hi.x
                x = np.full(per, lo[0] if face == 0 else hi[0]); z = lo[2] + s * (hi[2] - lo[2])
                out = np.array([-1.0, 0, 0]) if face == 0 else np.array([1.0, 0, 0])
            else:             # walls z = lo.z / hi.z
                z = np.full(per, lo[2] if face == 2 else hi[2]); x = lo[0] + s * (hi[0] - lo[0])
                out = np.array([0, 0, -1.0]) if face == 2 else np.array([0, 0, 1.0])
            pts.append(np.stack([x, np.zeros(per), z], 1))
            w = -out[None, :] * rng.uniform(0.2, 1.0, (per, 1)) + np.array([[0, -1.0, 0]])
            w[:, [0, 2]] += rng.uniform(-0.2, 0.2, (per, 2)) * (out[[2, 0]] != 0)
            dd.append(w / np.linalg.norm(w, axis=1, keepdims=True))
    pts = np.concatenate(pts)[:n_contact]
    dd = np.concatenate(dd)[:n_contact]
    # terrain height under each point: a vertical FP64 query of the terrain alone
    tt = _terrain_only(tris, obj)
    down = np.zeros((len(pts), 8), np.float32)
    down[:, 0] = pts[:, 0]; down[:, 1] = 1e3; down[:, 2] = pts[:, 2]
    down[:, 4] = -1.0; down[:, 6] = 0.0; down[:, 7] = 1e5
    _, th, _ = pyoracle.closest_f64_brute(tt, down)
    pts[:, 1] = 1e3 - th
    tgt.append(pts); dirs.append(dd); lab.append(np.full(len(pts), 3))
    tgt, dirs, lab = np.concatenate(tgt), np.concatenate(dirs), np.concatenate(lab)
    o = (tgt - 30.0 * dirs).astype(np.float32)
    r = scenes.rays8(o, dirs.astype(np.float32), 1e-4, 1e4)
    return r, lab


def _terrain_only(tris, obj):
    t = tris[obj == 0].reshape(-1, 9)
    out = np.zeros((len(t), 12), np.float32)
    out[:, 0:3], out[:, 4:7], out[:, 8:11] = t[:, 0:3], t[:, 3:6], t[:, 6:9]
    out[:, 3] = 1.0
    return out


def brute_gaps(gt, rays8):
    """FP64 brute force over every triangle: (nearest index, t1, t2, relative
    gap (t2 - t1) / t1, inf without two hits)."""
    ptr, t1, t2 = pyoracle.closest_f64_brute(gt, rays8)
    with np.errstate(invalid="ignore", divide="ignore"):
        gap = np.where(np.isfinite(t2) & (ptr >= 0), (t2 - t1) / t1, np.inf)
    return ptr, t1, t2, gap


def windowed_second(t1, t2):
    """The re-test's t_second: t2 when it is at most t1 + |t1| 1e-5 (float64,
    each operation rounded), else +inf."""
    lim = t1 + np.abs(t1) * 1e-5
    return np.where(t2 <= lim, t2, np.inf)
