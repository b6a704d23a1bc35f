"""Autotuner of the traversal kernels' launch parameters.

Searches, for one workload on the current GPU, over
  * threads per CTA and the shared-memory share of each lane's traversal
    stack (the kernel shapes the library ships: (128, 32), (64, 32),
    (256, 16), (128, 16)),
  * the refill interval: traversal steps a warp takes between two queue
    refills (8 ... 128), i.e. the size of the per-warp ray tile,
  * persistent CTAs per SM (the kernel's occupancy, or half of it),
timing each candidate with CUDA events (median of a few repetitions after a
warm-up) and returning the fastest.  Results can be saved as JSON and fed
back as ae_rt_config fields.
"""
from __future__ import annotations

import itertools
import json
from pathlib import Path

SHAPES = [(128, 32), (64, 32), (256, 16), (128, 16)]
REFILLS = [8, 16, 32, 64, 128]
BLOCKS = [0, -2]        # 0: occupancy; negative: occupancy // -n (resolved by the caller's kernel)


def candidates(shapes=SHAPES, refills=REFILLS, blocks=(0,)):
    for (threads, smem), refill, bps in itertools.product(shapes, refills, blocks):
        yield {"threads_per_block": threads, "stack_entries_smem": smem, "refill_steps": refill,
               "blocks_per_sm": bps}


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


def tune(make_run, torch, space=None, reps: int = 5, log=None):
    """make_run(config) -> (run, cleanup).  Returns (best_config, best_ms,
    all results)."""
    results = []
    best, best_ms = None, float("inf")
    for cfg in (space if space is not None else candidates()):
        run, cleanup = make_run(cfg)
        try:
            ms = time_workload(run, torch, reps=reps)
        finally:
            cleanup()
        results.append({**cfg, "ms": ms})
        if log:
            log(f"autotune {cfg} -> {ms:.3f} ms")
        if ms < best_ms:
            best, best_ms = cfg, ms
    return best, best_ms, results


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
