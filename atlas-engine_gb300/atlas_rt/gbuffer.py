"""G-buffers in the engine's form for the screen-space passes (ae_rt_rtao,
ae_rt_reflections, ae_rt_rtgi) where no rasteriser supplies them: NDC depth
(the engine's `depth` texture), the octahedral view-space normal
(EncodeNormal, data/shader/common/normalencode.hsh:3-16) and the inverse
projection and view matrices (globalData.ipMatrix / ivMatrix).

`view_rays` gives the camera rays through the pixels that the passes
reconstruct positions at (pixel centres, or the offset sub-pixels of a
half-resolution buffer); `device_gbuffer` traces them with the library's
closest-hit traversal and fills the planes on the device."""
from __future__ import annotations

import numpy as np


def look_at(eye, target, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """World-to-view matrix (4x4, row-major, the camera looks down -z)."""
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, up)
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    V = np.eye(4)
    V[0, :3], V[1, :3], V[2, :3] = r, u, -f
    V[:3, 3] = -V[:3, :3] @ eye
    return V


def perspective(fovy_deg: float, aspect: float, near: float, far: float) -> np.ndarray:
    """View-to-clip matrix with depth 0 at `near` and 1 at `far`."""
    f = 1.0 / np.tan(np.radians(fovy_deg) / 2)
    P = np.zeros((4, 4))
    P[0, 0], P[1, 1] = f / aspect, f
    P[2, 2], P[2, 3] = far / (near - far), far * near / (near - far)
    P[3, 2] = -1.0
    return P


def encode_normal(n: np.ndarray) -> np.ndarray:
    """EncodeNormal (common/normalencode.hsh:3-16) of unit vectors (n, 3) -> (n, 2)."""
    n = n / np.abs(n).sum(axis=1, keepdims=True)
    x, y, z = n[:, 0].copy(), n[:, 1], n[:, 2].copy()
    low = y < 0
    ox, oz = x[low].copy(), z[low].copy()
    x[low] = np.where(ox >= 0, 1.0, -1.0) * (1.0 - np.abs(oz))
    z[low] = np.where(oz >= 0, 1.0, -1.0) * (1.0 - np.abs(ox))
    return np.stack([x, z], axis=1)


def view_rays(V: np.ndarray, P: np.ndarray, w: int, h: int, offset: np.ndarray | None = None):
    """Origins and unit directions (float64, (w*h, 3)) of the rays from the
    eye through the points whose depth the passes read: pixel centres, or,
    with `offset` (half resolution), (2*pixel + offset + 0.5) of the full
    buffer (ao/rtao.csh:66)."""
    inv_pv = np.linalg.inv(P @ V)
    py, px = np.mgrid[0:h, 0:w]
    px, py = px.reshape(-1).astype(np.float64), py.reshape(-1).astype(np.float64)
    if offset is not None:
        off = np.asarray(offset, np.uint8).reshape(-1)
        tx, ty = (2 * px + (off & 1) + 0.5) / (2 * w), (2 * py + (off >> 1) + 0.5) / (2 * h)
    else:
        tx, ty = (px + 0.5) / w, (py + 0.5) / h
    ndc = np.stack([2 * tx - 1, 2 * ty - 1, np.ones_like(tx), np.ones_like(tx)], axis=1)
    far = ndc @ inv_pv.T
    far = far[:, :3] / far[:, 3:]
    eye = np.linalg.inv(V)[:3, 3]
    o = np.tile(eye, (len(far), 1))
    d = far - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d


def device_gbuffer(ctx, shading, V: np.ndarray, P: np.ndarray, w: int, h: int, half_res: bool = False,
                   seed: int = 3, device="cuda"):
    """A G-buffer of the context's scene (one identity-transform instance of
    the mesh whose GPUTriangle array is `shading`) as a dict of device
    tensors for Context.rtao / reflections / rtgi: the eye rays traced with
    ae_rt_trace_scene_closest, depth = the hit's NDC depth (1 where nothing
    is hit), normal = the encoded view-space face normal facing the eye."""
    import torch
    from . import scenes
    rng = np.random.default_rng(seed)
    offset = rng.integers(0, 4, w * h).astype(np.uint8) if half_res else None
    o, d = view_rays(V, P, w, h, offset)
    rays = torch.from_numpy(scenes.pack_rays(o.astype(np.float32), d.astype(np.float32))).to(device)
    n = w * h
    hits = torch.empty((n, 8), dtype=torch.float32, device=device)
    ctx.trace_scene_closest(rays, 0.0, 1e12, out=hits, n_rays=n)
    ctx.synchronize()
    t = hits[:, 0].double()
    tri = hits[:, 1].contiguous().view(torch.int32).long()
    hit = tri >= 0
    od = torch.from_numpy(o).to(device), torch.from_numpy(d).to(device)
    pos = od[0] + od[1] * t[:, None]
    pv = torch.from_numpy(P @ V).to(device)
    clip = torch.cat([pos, torch.ones_like(t)[:, None]], 1) @ pv.T
    depth = torch.where(hit, clip[:, 2] / clip[:, 3], torch.ones_like(t))
    sh = torch.as_tensor(shading, device=device).reshape(-1, 24)[tri.clamp(min=0)].double()
    nrm = torch.linalg.cross(sh[:, 4:7] - sh[:, 0:3], sh[:, 8:11] - sh[:, 0:3])
    nrm = nrm / (nrm.norm(dim=1, keepdim=True) + 1e-30)
    nrm = torch.where(((nrm * od[1]).sum(1, keepdim=True) > 0), -nrm, nrm)
    nv = nrm @ torch.from_numpy(V[:3, :3]).to(device).T
    nv = nv / (nv.norm(dim=1, keepdim=True) + 1e-30)
    enc = torch.from_numpy(encode_normal(nv.cpu().numpy())).to(device)
    enc = torch.where(hit[:, None], enc, torch.zeros_like(enc))
    gb = {"depth": depth.float().reshape(h, w).contiguous(), "normal": enc.float().reshape(h, w, 2).contiguous(),
          "half_res": int(half_res), "ip_matrix": np.linalg.inv(P), "iv_matrix": np.linalg.inv(V)}
    if half_res:
        gb["offset"] = torch.from_numpy(offset.reshape(h, w)).to(device)
    return gb
