"""Launch-shape autotuner for the orbit-integration kernels.

Times full calls of the integration under each candidate launch shape
(threads per block, blocks per SM, register variant of the Milky Way kernel)
with CUDA events on the launching stream and installs the fastest through
``gal_set_launch``. Results never depend on the launch shape (the device work
queue hands whole orbits to lanes), so tuning only changes speed.

Batches with very uneven orbit lengths end in a tail where the longest orbits
run almost alone; their speed then depends on which warps share a
sub-partition with them. A GB300 FP64 warp instruction holds its
sub-partition's FP64 pipe for ~64 cycles whatever the number of active lanes,
so one resident warp per sub-partition lets the longest orbits advance at their
own latency from the start. Shapes with many resident warps vary by up to 2x
from run to run. Each candidate is therefore timed ``repeats`` times and ranked
by its slowest run.
"""

from __future__ import annotations

from typing import Callable, Iterable

from . import _lib

DEFAULT_CANDIDATES = (
    # (block_threads, blocks_per_sm, variant); blocks_per_sm 0 = as many as fit.
    # One warp per SM sub-partition (128 x 1, 64 x 2) keeps a long orbit's FP64
    # instructions from queueing behind a second warp's: uneven batches end with
    # their longest orbits running alone, and their serial latency sets the time.
    (128, 1, 2),
    (64, 2, 2),
    (128, 1, 0),
    (128, 0, 2),
    (128, 0, 0),
)


def set_launch(method: int, adaptive: bool, block: int, per_sm: int, variant: int) -> None:
    L = _lib.load()
    _lib.check(L.gal_set_launch(int(method), int(bool(adaptive)), int(block), int(per_sm), int(variant)),
               "gal_set_launch")


# SMs given to four-warp teams for the longest orbits (second pass of a
# two-pass adaptive Milky Way batch, gal_set_team), per method. On the
# 262,144-orbit headline batch the step time has a narrow minimum, so the
# candidates are spaced closely around it (ms, Dopri5: 24 -> 1,253,
# 28 -> 1,171, 30 -> 1,172, 32 -> 1,183, 36 -> 1,211, 40 -> 1,241; Dopri8:
# 2 -> 1,590, 4 -> 1,525, 6 -> 1,500, 8 -> 1,454, 12 -> 1,474, 16 -> 1,499,
# 24 -> 1,549, 32 -> 1,609, none -> 1,852).
DEFAULT_TEAMS = {5: (24, 28, 32, 40), 8: (6, 8, 10, 12, 16)}


def set_team(blocks: int) -> None:
    L = _lib.load()
    _lib.check(L.gal_set_team(int(blocks)), "gal_set_team")


# Fraction of every orbit's span covered by the first pass of the two-pass
# schedule (gal_set_split_fraction; the library's default is 0.1). The first
# pass's progress is what orders the second pass longest first: too short a
# first pass misorders the longest orbits (headline batch, 28 team SMs, ms:
# 0.06 -> 1,243-1,251, 0.08 -> 1,156, 0.1 -> 1,171, 0.13 -> 1,192).
DEFAULT_SPLITS = (0.08, 0.1, 0.12)


def set_split_fraction(frac: float) -> None:
    L = _lib.load()
    _lib.check(L.gal_set_split_fraction(float(frac)), "gal_set_split_fraction")


def _worst_ms(run: Callable[[], object], repeats: int) -> float:
    import torch

    stream = torch.cuda.current_stream()
    worst = 0.0
    for _ in range(repeats):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        torch.cuda.synchronize()
        worst = max(worst, e0.elapsed_time(e1))
    return worst


def tune(run: Callable[[], object], method: int, adaptive: bool,
         candidates: Iterable[tuple[int, int, int]] = DEFAULT_CANDIDATES, repeats: int = 2,
         teams: Iterable[int] | None = None, splits: Iterable[float] = DEFAULT_SPLITS) -> dict:
    """Run ``run()`` under each launch-shape candidate ``repeats`` times and keep
    the one whose slowest run is fastest (no candidates: the shape is left as
    it is); then, for adaptive batches, the same over the number of SMs given to
    four-warp teams (``teams``, by default the method's candidates) and, with the
    best of those, over the first pass's split fraction. Returns the timings."""
    timings = {}
    for cand in candidates:
        set_launch(method, adaptive, *cand)
        timings[cand] = _worst_ms(run, repeats)
    out = {"best": {}, "ms": {}}
    if timings:
        best = min(timings, key=timings.get)
        set_launch(method, adaptive, *best)
        out = {"best": {"block_threads": best[0], "blocks_per_sm": best[1], "variant": best[2]},
               "ms": {f"{b}x{s}v{v}": round(t, 3) for (b, s, v), t in timings.items()}}
    if teams is None:
        teams = DEFAULT_TEAMS.get(method, ()) if adaptive else ()
    if adaptive and teams:
        tt = {}
        for blocks in teams:
            set_team(blocks)
            tt[blocks] = _worst_ms(run, repeats)
        tbest = min(tt, key=tt.get)
        set_team(tbest)
        out["best"]["team_blocks"] = tbest
        out["team_ms"] = {str(k): round(v, 3) for k, v in tt.items()}
        if splits:
            sp = {}
            for frac in splits:
                set_split_fraction(frac)
                sp[frac] = _worst_ms(run, repeats)
            fbest = min(sp, key=sp.get)
            set_split_fraction(fbest)
            out["best"]["split_fraction"] = fbest
            out["split_ms"] = {str(k): round(v, 3) for k, v in sp.items()}
    return out
