"""Launch-schedule autotuner for the batched frame.

The schedule (tc_schedule) sets the launch shapes of the persistent stages:
grid multipliers of the classify warp kernels and of the instantiate
allocation, the vertex kernel's register budget, the grid of the
full-cluster vertex kernel (which runs beside the rest of the frame), the
split tile size
(128 threads x 16 items, 256 or 512 threads x 32 items), the split grid, and
the frame graph's shape (the first part run allocated beside the split passes,
or every run after them) and the split passes' form (one launch, or one per
pass).
Outputs do not depend on it (every allocation is a prefix sum in a fixed
order), so tuning is a pure timing search.

Search: coordinate descent from the current schedule; each candidate is timed
as the mean CUDA-event duration of whole graph frames over the caller's
frames (three passes), with L2 flushed before each frame. Two sweeps over the parameters
usually settle; each trial re-captures the frame graph once.

    best, report = autotune(pipe, frames, set_frame, flush)
    pipe.set_schedule(best)
"""
from __future__ import annotations

import statistics

SPACE = {
    "classifyBlocksPerSM": (4, 6, 8, 16),
    "scanBlocksPerSM": (1, 2, 4, 8, 16),
    "splitBlockSize": (128, 256, 512),
    "blocksPerSM": (1, 2, 4),
    "vertexBlocksPerSM": (3, 4, 5, 6),
    "fullVertexBlocksPerSM": (1, 2, 3, 4),
    "vertexGridPerSM": (0, 1, 2, 3, 8, 16),
    "frameShape": (0, 1),
    "splitPerPass": (0, 1),
}


def time_schedule(pipe, sched: dict, frames, set_frame, flush, reps: int = 1) -> float:
    """Mean graph-frame time (ms) of `sched` over `frames` x `reps` (the mean,
    not the median: frame throughput is total triangles over total time, so
    a schedule's slow frames count as much as its typical one)."""
    torch = pipe.torch
    pipe.set_schedule(sched)
    set_frame(frames[0])
    pipe.build("graph")  # capture outside the timing
    ts = []
    for _ in range(reps):
        for f in frames:
            set_frame(f)
            flush()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            pipe.build("graph")
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
    return statistics.mean(ts)


def autotune(pipe, frames, set_frame, flush, space: dict | None = None, sweeps: int = 2, reps: int = 3):
    """Coordinate descent over `space`; returns (best schedule, report)."""
    space = dict(space or SPACE)
    start = pipe.schedule()
    best = dict(start)
    cache: dict[tuple, float] = {}

    def measure(s):
        key = tuple(sorted(s.items()))
        if key not in cache:
            cache[key] = time_schedule(pipe, s, frames, set_frame, flush, reps)
        return cache[key]

    base_ms = measure(best)
    best_ms = base_ms
    for _ in range(sweeps):
        improved = False
        for name, values in space.items():
            for v in values:
                if v == best[name]:
                    continue
                cand = dict(best, **{name: v})
                ms = measure(cand)
                if ms < best_ms * 0.99:  # ignore sub-1% noise
                    best, best_ms, improved = cand, ms, True
        if not improved:
            break
    pipe.set_schedule(best)
    report = {"start": start, "start_ms": base_ms, "best": best, "best_ms": best_ms, "trials": len(cache),
              "frames": len(frames)}
    return best, report
