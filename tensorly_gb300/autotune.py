"""Autotuner for the batched CP-ALS kernel variants.

``tlgb_cp_als_batched`` sorts the tensors of a batch into three size classes
(by the shared-memory footprint of the padded tensor) and runs each class with
a kernel variant of 128, 256 or 512 threads per CTA (4, 2 or 1 CTAs per SM).
``tune_batched`` times every variant for every class on the caller's own batch
(a few sweeps, CUDA events, the other classes left at their current choice),
keeps the fastest, sets it with ``tlgb_set_tuning`` and returns the choice.
Choices are cached per device and batch signature for the process.
"""

import ctypes

import torch

from . import _lib

CLASSES = ("small", "medium", "large")
VARIANTS = (128, 256, 512)
_cache = {}


def _set(cls, nt):
    _lib.check(_lib.lib().tlgb_set_tuning(f"batched_threads_{cls}".encode(), int(nt)))


def _time(problem, sweeps, reps):
    st = torch.cuda.current_stream()
    problem.run(sweeps)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(reps):
        problem.run(sweeps)
    b.record(st)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def tune_batched(problem, sweeps=4, reps=2, verbose=False):
    """Pick the fastest variant per size class for ``problem`` (a
    ``BatchedProblem``); returns {class: threads} and leaves it set."""
    key = (torch.cuda.get_device_name(problem.device), len(problem),
           tuple(sorted(set(problem.shapes)))[:64], tuple(problem.ranks[:64]))
    if key in _cache:
        for cls, nt in _cache[key].items():
            _set(cls, nt)
        return dict(_cache[key])
    choice = {cls: 0 for cls in CLASSES}
    for cls in CLASSES:
        best = None
        for nt in VARIANTS:
            _set(cls, nt)
            ms = _time(problem, sweeps, reps)
            if verbose:
                print(f"batched {cls}: {nt} threads -> {ms:.2f} ms")
            if best is None or ms < best[0]:
                best = (ms, nt)
        choice[cls] = best[1]
        _set(cls, best[1])
    _cache[key] = dict(choice)
    return choice


def reset_batched():
    """Back to the library defaults (128 / 256 / 512)."""
    for cls in CLASSES:
        _set(cls, 0)
