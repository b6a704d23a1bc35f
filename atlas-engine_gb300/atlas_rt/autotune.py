"""Autotuner of the traversal kernels' launch parameters.

Searches, for one workload on the current GPU, the axes
  * shape: threads per CTA and the shared-memory share of each lane's
    traversal stack (the kernel shapes the library ships: (128, 32),
    (64, 32), (256, 16), (128, 16));
  * refill_steps: traversal steps a warp takes between two queue refills,
    i.e. the size of the per-warp ray tile (8 ... 64);
  * refill_below: refill as soon as fewer lanes than this still traverse
    (never, 8, 16, 24);
  * leaf_wait: closest-hit lanes at a leaf wait for this many leaf lanes
    (0, 2, 4, 6);
  * workload-specific axes (for the path tracer: the number of image tiles,
    which sets the size of its wavefront queues);
by coordinate descent: starting from the library's defaults, each axis in
turn is swept with the others fixed and the fastest value kept, until a pass
changes nothing (at most `passes` passes).  Each candidate is timed with CUDA
events (median of a few repetitions after a warm-up).  The result is saved as
JSON (atlas_rt/tuning.json) and fed back as ae_rt_config fields.
"""
from __future__ import annotations

import json
from pathlib import Path

SHAPES = [(128, 32), (64, 32), (256, 16), (128, 16)]
AXES = {
    "shape": SHAPES,
    "refill_steps": [8, 16, 32, 64],
    "refill_below": [33, 8, 16, 24],      # 33: never refill early
    "leaf_wait": [0, 2, 4, 6],
}
DEFAULTS = {"shape": (128, 32), "refill_steps": 32, "refill_below": 8, "leaf_wait": 0}
CONFIG_KEYS = ("threads_per_block", "stack_entries_smem", "refill_steps", "refill_below", "leaf_wait",
               "blocks_per_sm")


def to_config(point: dict) -> dict:
    """A search point as Context keyword arguments (other axes are the
    workload's own)."""
    cfg = {k: v for k, v in point.items() if k != "shape"}
    if "shape" in point:
        cfg["threads_per_block"], cfg["stack_entries_smem"] = point["shape"]
    return cfg


def context_kwargs(cfg: dict | None) -> dict:
    """The ae_rt_config fields of a tuned configuration."""
    return {k: v for k, v in (cfg or {}).items() if k in CONFIG_KEYS}


def time_workload(run, torch, reps: int = 5, warmup: int = 2) -> float:
    """Median milliseconds of run() measured with CUDA events."""
    for _ in range(warmup):
        run()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        run()
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    ts.sort()
    return ts[len(ts) // 2]


def search(make_run, torch, axes=None, start=None, reps: int = 5, passes: int = 2, log=None):
    """Coordinate descent.  make_run(config) -> (run, cleanup).  Returns
    (best_config, best_ms, every timed point)."""
    axes = dict(AXES if axes is None else axes)
    point = dict(DEFAULTS if start is None else start)
    point = {k: v for k, v in point.items() if k in axes}
    results, cache = [], {}

    def measure(p):
        key = json.dumps(p, sort_keys=True, default=list)
        if key not in cache:
            cfg = to_config(p)
            run, cleanup = make_run(cfg)
            try:
                cache[key] = time_workload(run, torch, reps=reps)
            finally:
                cleanup()
            results.append({**cfg, "ms": cache[key]})
            if log:
                log(f"autotune {cfg} -> {cache[key]:.3f} ms")
        return cache[key]

    best_ms = measure(point)
    for _ in range(passes):
        changed = False
        for axis, values in axes.items():
            for v in values:
                cand = {**point, axis: v}
                if cand == point:
                    continue
                ms = measure(cand)
                if ms < best_ms * 0.995:       # a change must win by more than the noise
                    point, best_ms, changed = cand, ms, True
        if not changed:
            break
    return to_config(point), best_ms, results


def save(path: Path, workload: str, best: dict, best_ms: float, results: list, gpu: str):
    path = Path(path)
    data = json.loads(path.read_text()) if path.exists() else {}
    data[workload] = {"gpu": gpu, "best": best, "best_ms": best_ms, "results": results}
    path.write_text(json.dumps(data, indent=1) + "\n")


def load(path: Path, workload: str):
    path = Path(path)
    if not path.exists():
        return None
    return json.loads(path.read_text()).get(workload, {}).get("best")
