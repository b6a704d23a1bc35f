"""The engine's NEE light list on the host (libatlas_rt.so's ae_lights_*):
triangle lights of a mesh (RayTracingWorld::BuildTriangleLightsForMesh,
RayTracingWorld.cpp:322-376), their placement per instance
(UpdateTriangleLights, :378-407), directional lights and the weight
normalisation (RayTracingHelper::UpdateLights, RayTracingHelper.cpp:436-500)
and the per-dispatch selection of at most 128 lights (DispatchAndHit,
RayTracingHelper.cpp:72-105).  Records are (n, 16) float32 GPULight rows."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._native import AeRtError, lib

ENGINE_LIGHT_CAPACITY = 128     # RayTracingHelper.cpp:20


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _check(st):
    if st != 0:
        raise AeRtError(st, "light list")


def from_mesh(shading: np.ndarray, emissive_srgb, emissive_intensity) -> np.ndarray:
    """One GPULight per emissive triangle of a GPUTriangle array (n, 24)."""
    sh = np.ascontiguousarray(shading, np.float32).reshape(-1, 24)
    em = np.ascontiguousarray(emissive_srgb, np.float32).reshape(-1, 3)
    it = np.ascontiguousarray(emissive_intensity, np.float32).reshape(-1)
    n = C.c_uint32()
    _check(lib().ae_lights_from_mesh(_p(sh), len(sh), _p(em), _p(it), len(em), None, 0, C.byref(n)))
    out = np.zeros((n.value, 16), np.float32)
    _check(lib().ae_lights_from_mesh(_p(sh), len(sh), _p(em), _p(it), len(em), _p(out), n.value, C.byref(n)))
    return out


def instance(mesh_lights: np.ndarray, model, instance_index: int) -> np.ndarray:
    L = np.ascontiguousarray(mesh_lights, np.float32).reshape(-1, 16)
    M = np.ascontiguousarray(model, np.float32).reshape(4, 4)
    out = np.zeros_like(L)
    _check(lib().ae_lights_instance(_p(L), len(L), _p(M), int(instance_index), _p(out)))
    return out


def directional(color_srgb, intensity: float, direction, index: int = 0) -> np.ndarray:
    c = np.ascontiguousarray(color_srgb, np.float32)
    d = np.ascontiguousarray(direction, np.float32)
    out = np.zeros(16, np.float32)
    _check(lib().ae_light_directional(_p(c), float(intensity), _p(d), int(index), _p(out)))
    return out


def normalize(lights: np.ndarray) -> np.ndarray:
    L = np.ascontiguousarray(lights, np.float32).reshape(-1, 16).copy()
    _check(lib().ae_lights_normalize(_p(L), len(L)))
    return L


def select(lights: np.ndarray, capacity: int = ENGINE_LIGHT_CAPACITY, uniforms=None, seed: int = 0) -> np.ndarray:
    """At most `capacity` lights for one dispatch; draws use `uniforms`
    (capacity floats in [0, 1)) or a numpy generator seeded with `seed`."""
    L = np.ascontiguousarray(lights, np.float32).reshape(-1, 16)
    u = None
    if len(L) > capacity:
        u = (np.random.default_rng(seed).random(capacity, dtype=np.float32) if uniforms is None
             else np.ascontiguousarray(uniforms, np.float32))
        if len(u) < capacity:
            raise ValueError("need one uniform per selected light")
    out = np.zeros((min(len(L), capacity), 16), np.float32)
    n = C.c_uint32()
    _check(lib().ae_lights_select(_p(L), len(L), capacity, _p(u), _p(out), C.byref(n)))
    return out[: n.value]
