"""Launch-shape autotuner for the orbit-integration kernels.

Times one full call of the integration under each candidate launch shape
(threads per block, blocks per SM, register variant of the Milky Way kernel)
with CUDA events on the launching stream and installs the fastest through
``gal_set_launch``. Results never depend on the launch shape (the device work
queue hands whole orbits to lanes), so tuning only changes speed.
"""

from __future__ import annotations

from typing import Callable, Iterable

from . import _lib

DEFAULT_CANDIDATES = (
    # (block_threads, blocks_per_sm, variant)
    (128, 0, 0),
    (128, 0, 1),
    (64, 0, 0),
    (128, 0, 2),
)


def set_launch(method: int, adaptive: bool, block: int, per_sm: int, variant: int) -> None:
    L = _lib.load()
    _lib.check(L.gal_set_launch(int(method), int(bool(adaptive)), int(block), int(per_sm), int(variant)),
               "gal_set_launch")


def tune(run: Callable[[], object], method: int, adaptive: bool,
         candidates: Iterable[tuple[int, int, int]] = DEFAULT_CANDIDATES, repeats: int = 1) -> dict:
    """Run ``run()`` under each candidate, keep the fastest; returns the timings."""
    import torch

    timings = {}
    for cand in candidates:
        set_launch(method, adaptive, *cand)
        torch.cuda.synchronize()
        stream = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(repeats):
            run()
        e1.record(stream)
        torch.cuda.synchronize()
        timings[cand] = e0.elapsed_time(e1) / repeats
    best = min(timings, key=timings.get)
    set_launch(method, adaptive, *best)
    return {"best": {"block_threads": best[0], "blocks_per_sm": best[1], "variant": best[2]},
            "ms": {f"{b}x{s}v{v}": round(t, 3) for (b, s, v), t in timings.items()}}
