"""Autotuners for the CP-ALS kernels.

Dense tensor-core MTTKRP (``tune_dense``): the tile shape along the
contracted modes (the inner-mode group whose slice of the split factor stays
resident in shared memory, ``tc_group_kib``), the depth of the tensor-tile
ring (``tc_stages``) and the grid (``tc_waves`` waves of one CTA per SM) are
searched coordinate by coordinate on the caller's own tensor: each candidate
runs a few bf16 sweeps of ``parafac`` (CUDA events), the fastest is kept and
set with ``tlgb_set_tuning``.

Batched CP-ALS kernel variants (``tune_batched``):

``tlgb_cp_als_batched`` sorts the tensors of a batch into three size classes
(by the shared-memory footprint of the padded tensor) and runs each class with
a kernel variant of 128, 256 or 512 threads per CTA (4, 2 or 1 CTAs per SM)
and an MTTKRP work tile of one row, four rank columns and ``outer_tile``
slices of the outer mode (0: the slices spread over as many groups as there
are threads).  ``tune_batched`` times, per class, every thread count and then
every outer tile on the caller's own batch (a few sweeps, CUDA events, the
other classes left at their current choice), keeps the fastest, sets it with
``tlgb_set_tuning`` and returns the choice.  Choices are cached per device
and batch signature for the process.
"""

import ctypes

import torch

from . import _lib

CLASSES = ("small", "medium", "large")
VARIANTS = (128, 256, 512)
OUTER_TILES = (0, 2, 4, 8, 16)
_cache = {}


def _set(cls, nt):
    _lib.check(_lib.lib().tlgb_set_tuning(f"batched_threads_{cls}".encode(), int(nt)))


def _set_tile(cls, ot):
    _lib.check(_lib.lib().tlgb_set_tuning(f"batched_outer_tile_{cls}".encode(), int(ot)))


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
    """Pick the fastest thread count, then the fastest MTTKRP outer tile, per
    size class for ``problem`` (a ``BatchedProblem``); returns {class:
    threads} and {class: outer_tile} and leaves them set."""
    key = (torch.cuda.get_device_name(problem.device), len(problem),
           tuple(sorted(set(problem.shapes)))[:64], tuple(problem.ranks[:64]))
    if key in _cache:
        threads, tiles = _cache[key]
        for cls in CLASSES:
            _set(cls, threads[cls])
            _set_tile(cls, tiles[cls])
        return dict(threads), dict(tiles)
    threads = {cls: 0 for cls in CLASSES}
    tiles = {cls: 0 for cls in CLASSES}
    for cls in CLASSES:
        _set_tile(cls, 0)
        best = None
        for nt in VARIANTS:
            _set(cls, nt)
            ms = _time(problem, sweeps, reps)
            if verbose:
                print(f"batched {cls}: {nt} threads -> {ms:.2f} ms")
            if best is None or ms < best[0]:
                best = (ms, nt)
        threads[cls] = best[1]
        _set(cls, best[1])
        for ot in OUTER_TILES[1:]:
            _set_tile(cls, ot)
            ms = _time(problem, sweeps, reps)
            if verbose:
                print(f"batched {cls}: outer tile {ot} -> {ms:.2f} ms")
            if ms < best[0]:
                best = (ms, best[1])
                tiles[cls] = ot
        _set_tile(cls, tiles[cls])
    _cache[key] = (dict(threads), dict(tiles))
    return threads, tiles


def reset_batched():
    """Back to the library defaults (128 / 256 / 512 threads, default tiles)."""
    for cls in CLASSES:
        _set(cls, 0)
        _set_tile(cls, 0)


DENSE_SPACE = (
    ("tc_group_kib", (32, 48, 64, 96)),
    ("tc_stages", (0, 5, 7, 9)),      # 0: as deep as shared memory allows
    ("tc_waves", (1, 2)),
)
DENSE_DEFAULT = {"tc_group_kib": 64, "tc_stages": 0, "tc_waves": 1}
_dense_cache = {}


def _set_key(key, value):
    _lib.check(_lib.lib().tlgb_set_tuning(key.encode(), int(value)))


def _time_dense(x, rank, init, sweeps, reps, refine_sweeps):
    from .cp_tensor import CPTensor
    from .decomposition import parafac

    def run():
        parafac(x, rank, init=CPTensor((None, [f.clone() for f in init])), n_iter_max=sweeps,
                tol=0, precision="bf16", refine_sweeps=refine_sweeps)
    run()
    st = torch.cuda.current_stream()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(reps):
        run()
    b.record(st)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def tune_dense(x, rank, sweeps=50, refine_sweeps=1, reps=2, min_gain=0.01, verbose=False):
    """Pick the tensor-core MTTKRP's inner-mode group size, ring depth and
    wave count for bf16 CP-ALS of the f32 CUDA tensor ``x`` at ``rank`` by a
    coordinate search over ``DENSE_SPACE`` (the defaults first); a value
    replaces the current one only if it is at least ``min_gain`` faster, so
    timing noise does not move the choice.  Each candidate is timed on whole
    ``parafac`` calls of ``sweeps`` sweeps, the last ``refine_sweeps`` of them
    f32 closing sweeps (the tile choice also sets their three-plane plans),
    so the mix is that of the run being tuned.  Returns {key: value} and
    leaves it set.  Cached per device, shape, rank and sweep mix."""
    key = (torch.cuda.get_device_name(x.device), tuple(x.shape), int(rank), int(sweeps),
           int(refine_sweeps))
    if key in _dense_cache:
        for k, v in _dense_cache[key].items():
            _set_key(k, v)
        return dict(_dense_cache[key])
    gen = torch.Generator(device="cpu").manual_seed(0)
    init = [torch.rand((int(s), int(rank)), generator=gen).to(x.device, torch.float32)
            for s in x.shape]
    choice = dict(DENSE_DEFAULT)
    for k, v in choice.items():
        _set_key(k, v)
    best_ms = _time_dense(x, rank, init, sweeps, reps, refine_sweeps)
    if verbose:
        print(f"dense defaults {choice}: {best_ms:.3f} ms")
    for k, values in DENSE_SPACE:
        for v in values:
            if v == choice[k]:
                continue
            _set_key(k, v)
            try:
                ms = _time_dense(x, rank, init, sweeps, reps, refine_sweeps)
            except NotImplementedError:     # the plan does not fit with this value
                ms = float("inf")
            if verbose:
                print(f"dense {k}={v}: {ms:.3f} ms")
            if ms < (1.0 - min_gain) * best_ms:
                best_ms, choice[k] = ms, v
        _set_key(k, choice[k])
    _dense_cache[key] = dict(choice)
    return choice


def reset_dense():
    """Back to the library's tensor-core MTTKRP defaults."""
    for k in DENSE_DEFAULT:
        _set_key(k, 0)
