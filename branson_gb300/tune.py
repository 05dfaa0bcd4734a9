"""Autotuner for the transport schedule of one deck.

The choices are the ones that change speed and never results: the history
kernel's block size (64, 128 or 256 threads), histories per thread (the
persistent grid: the occupancy grid or a half or a quarter of it, so each
thread takes 1x, 2x or 4x the histories), and history mode vs event mode
(stage rounds over sorted queues, with a history-kernel tail).  Each
candidate transports the same step of the caller's context -- the adjoint
forward without a tape, which sources and transports a copy of the step's
bank and leaves the context where it was -- a few times; the fastest median
kernel time wins and is applied to the context.  Every candidate must
reproduce the first one's tallies bit for bit (they are exact fixed-point
sums of the same histories); a difference raises.
"""
from __future__ import annotations

import statistics
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _lib
from .adjoint import step_forward
from .engine import ReplicatedIMC


@dataclass(frozen=True)
class Schedule:
    algorithm: int = _lib.HISTORY
    threads: int = 128
    grid_fraction: float = 1.0      # of the occupancy grid: 1/histories-per-thread multiplier
    event_round_cap: int = 64
    event_tail_fraction: float = 0.02

    def label(self) -> str:
        mode = "history" if self.algorithm == _lib.HISTORY else f"event(rounds<={self.event_round_cap})"
        return f"{mode} threads={self.threads} grid={self.grid_fraction:g}"


@dataclass
class TuneResult:
    best: Schedule
    best_ms: float
    timings: List[tuple] = field(default_factory=list)   # (Schedule, median ms)

    def speedup_over(self, s: Schedule) -> float:
        for c, ms in self.timings:
            if c == s:
                return ms / self.best_ms
        raise KeyError(s)


def default_candidates() -> List[Schedule]:
    out = [Schedule(_lib.HISTORY, t, g) for t in (64, 128, 256) for g in (1.0, 0.5, 0.25)]
    out += [Schedule(_lib.EVENT, 128, 1.0, cap) for cap in (8, 32)]
    return out


def apply(imc: ReplicatedIMC, s: Schedule, n_sm: int, blocks_per_sm: Optional[int] = None) -> None:
    """Set a schedule on a context (its step() then runs in the schedule's
    algorithm).  grid_fraction < 1 shrinks the occupancy grid (blocks_per_sm
    blocks per SM for the chosen block size)."""
    imc.algorithm = s.algorithm
    imc.set_option("transport_threads", s.threads)
    if s.grid_fraction >= 1.0 or blocks_per_sm is None:
        imc.set_option("transport_blocks", 0)
    else:
        imc.set_option("transport_blocks", max(1, int(round(n_sm * blocks_per_sm * s.grid_fraction))))
    imc.set_option("event_round_cap", s.event_round_cap)
    imc.set_option("event_tail_fraction", s.event_tail_fraction)


def _blocks_per_sm(threads: int) -> int:
    # the history kernel keeps the register budget of six 128-thread blocks
    # per SM for every block size (launch bounds in bgs_transport.cu)
    return max(1, (6 * 128) // threads)


def tune(imc: ReplicatedIMC, candidates: Optional[Sequence[Schedule]] = None, repeats: int = 3,
         n_sm: Optional[int] = None) -> TuneResult:
    """Time every candidate on the context's current step and apply the fastest."""
    if n_sm is None:
        import torch
        n_sm = torch.cuda.get_device_properties(imc.device).multi_processor_count
    cands = list(candidates) if candidates is not None else default_candidates()
    ref = None
    timings = []
    for c in cands:
        apply(imc, c, n_sm, _blocks_per_sm(c.threads))
        times = []
        for _ in range(repeats + 1):
            abs_E, _ = step_forward(imc, save=False, algorithm=c.algorithm)
            ms, _k = imc.last_transport_ms()
            times.append(ms)
            if ref is None:
                ref = abs_E
            elif not np.array_equal(abs_E, ref):
                raise RuntimeError(f"schedule {c.label()} changed the tallies: the transport is not order-independent")
        timings.append((c, statistics.median(times[1:])))
    best, best_ms = min(timings, key=lambda t: t[1])
    apply(imc, best, n_sm, _blocks_per_sm(best.threads))
    return TuneResult(best=best, best_ms=best_ms, timings=timings)
