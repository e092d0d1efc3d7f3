"""Tile autotuner for resample_poly (no MatX counterpart).

For one workload (input rows, filter, up/down) the tuner times every candidate
row-tile shape of the resample kernel on the device with CUDA events and keeps
the fastest:

  rows_per_thread (outputs per thread along the row direction)  1, 2, 4
  col_warps       (phases per CTA = 8 * col_warps per pass)     1, 2, 4, 8; 9..16 dividing
                                                                the super-groups (one row slice,
                                                                1 or 2 rows per thread)
  group           (outputs per tile row = group * up)           multiples giving up*group % 4 == 0
  buffers         (prefetch the next input window or not)       1, 2; plus 4 to send the
                                                                outputs through shared memory
                                                                and TMA tensor stores (complex
                                                                float signal, real taps)

The winner is registered in the library (gbfir_resample_tile_register), so every
later call with the same reduced (up, down) and filter length uses it, and it is
stored in a JSON cache keyed by device name, dtype, rates, filter length and the
row-length bucket, so a later process can register it without re-timing.

``tune_ragged`` does the same for the ragged launch: per reduced (up, down) and
tap-length bucket (the smallest power of two >= the tap count) it times the ragged
launch of that group's signals under every candidate shape (rows per thread 1 or 2,
column warps 1/2/4/8, row groups of 1, 2 or 4 times the smallest) and registers the
winner with gbfir_ragged_tile_register, which later ragged plans read.
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import dataclass, field

import torch

from . import _lib
from . import resample_poly, set_resample_tile

CACHE = os.environ.get("MATX_GB300_TUNE_CACHE",
                       os.path.join(os.path.expanduser("~"), ".cache", "matx_gb300", "resample_tiles.json"))


@dataclass
class TuneResult:
    key: str
    best: tuple
    best_ms: float
    default_ms: float
    table: list = field(default_factory=list)


def _key(x: torch.Tensor, h: torch.Tensor, up: int, down: int) -> str:
    g = math.gcd(up, down)
    name = torch.cuda.get_device_name(x.device).replace(" ", "_")
    nbucket = 1 << max(0, int(math.log2(max(1, x.shape[-1]))))
    return f"{name}|{x.dtype}|{h.dtype}|{up // g}/{down // g}|L{h.shape[-1]}|N{nbucket}|B{x.numel() // x.shape[-1]}"


def candidates(up: int, down: int, tma_store: bool = False):
    g = math.gcd(up, down)
    # complex float signals with real taps: also the ring form (3), the TMA-store epilogue (+4)
    # and, where the row stride down*group is even, the paired walk (+8)
    base = (1, 2, 3, 5, 6, 7) if tma_store else (1, 2)

    def nbufs_for(grp):
        if tma_store and ((down // g) * grp) % 2 == 0:
            return base + (9, 10, 11, 13, 14, 15)
        return base
    u = up // g
    g0 = 4 // math.gcd(u, 4)
    # odd multiples too: they keep an odd row stride (TMA window copies) for odd down
    groups = sorted({g0 * m for m in (1, 2, 3, 4, 5, 7, 8) if g0 * m <= 64})
    for rq in (1, 2, 4):
        for wc in (1, 2, 4, 8):
            for grp in groups:
                nsg = (u * grp + 7) // 8
                if wc > max(1, nsg):
                    continue
                for nb in nbufs_for(grp):
                    yield (rq, wc, grp, nb)
    # one row slice of 9..16 column warps that divide the super-groups evenly (one or two
    # rows per thread): balanced warps where 1, 2, 4 or 8 leave some with an extra super-group
    for grp in groups:
        nsg = (u * grp + 7) // 8
        for wc in range(9, 17):
            if nsg % wc == 0:
                for rq in (1, 2):
                    for nb in nbufs_for(grp):
                        yield (rq, wc, grp, nb)


def _time(fn, reps: int) -> float:
    """Median device time of fn over reps launches.  A ~50 us device-side delay before each
    start event keeps the GPU busy while the host dispatches fn, so the host's dispatch
    latency (tens of microseconds, and noisy) stays out of the comparison."""
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        torch.cuda._sleep(100_000)
        start.record()
        fn()
        stop.record()
        stop.synchronize()
        ts.append(start.elapsed_time(stop))
    ts.sort()
    return ts[len(ts) // 2]


def register(up: int, down: int, h_len: int, tile) -> None:
    rq, wc, grp, nb = tile
    _lib.check(_lib.load().gbfir_resample_tile_register(up, down, h_len, rq, wc, grp, nb))


def load_cache() -> dict:
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save_cache(d: dict) -> None:
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        tmp = CACHE + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, CACHE)
    except OSError:
        pass


def tune_resample(x: torch.Tensor, h: torch.Tensor, up: int, down: int, *, reps: int = 5,
                  out: torch.Tensor | None = None, use_cache: bool = True) -> TuneResult:
    """Time all candidate tiles on (x, h) and register the fastest."""
    key = _key(x, h, up, down)
    cache = load_cache() if use_cache else {}
    if key in cache:
        ent = cache[key]
        tile = tuple(ent["best"])
        register(up, down, h.shape[-1], tile)
        return TuneResult(key, tile, ent["best_ms"], ent["default_ms"], [])
    if out is None:
        out = resample_poly(x, h, up, down)
    run = lambda: resample_poly(x, h, up, down, out=out)
    set_resample_tile(0, 0, 0, 0)
    default_ms = _time(run, reps)
    table = []
    try:
        tma_store = x.dtype == torch.complex64 and not h.is_complex()
        for tile in candidates(up, down, tma_store):
            set_resample_tile(*tile)
            try:
                ms = _time(run, reps)
            except _lib.GbfirError:
                continue
            table.append((tile, ms))
        # the closest few again, with more launches each, so noise does not pick the tile
        table.sort(key=lambda t: t[1])
        final = []
        for tile, _ in table[:6]:
            set_resample_tile(*tile)
            final.append((tile, _time(run, 3 * reps)))
    finally:
        set_resample_tile(0, 0, 0, 0)
    best, best_ms = min(final, key=lambda t: t[1])
    register(up, down, h.shape[-1], best)
    if use_cache:
        cache[key] = {"best": list(best), "best_ms": best_ms, "default_ms": default_ms}
        _save_cache(cache)
    return TuneResult(key, best, best_ms, default_ms, table)


def _bucket(n: int) -> int:
    b = 1
    while b < n:
        b <<= 1
    return b


def ragged_candidates(up: int, down: int):
    g = math.gcd(up, down)
    u = up // g
    g0 = 4 // math.gcd(u, 4)
    for rq in (1, 2):
        for wc in (1, 2, 4, 8):
            for m in (1, 2, 4):
                if g0 * m <= 64:
                    yield (rq, wc, g0 * m)


def tune_ragged(signals, *, reps: int = 3, max_per_group: int = 64) -> dict:
    """Tune the ragged launch's tile shape per (reduced up/down, tap-length bucket) group of
    ``signals`` ((x, h, up, down) tuples as for RaggedPlan): each group's longest signals are
    planned and launched alone under every candidate shape; the fastest shape (or the
    built-in heuristic, if nothing beats it) is registered for later plans."""
    from .ragged import RaggedPlan
    lib = _lib.load()
    groups = {}
    for x, h, up, down in signals:
        g = math.gcd(int(up), int(down))
        u, d = int(up) // g, int(down) // g
        if u == d:
            continue
        groups.setdefault((u, d, _bucket(h.shape[-1])), []).append((x, h, up, down))
    results = {}
    for (u, d, b), sigs in sorted(groups.items()):
        sigs = sorted(sigs, key=lambda s: -s[0].shape[-1])[:max_per_group]
        _lib.check(lib.gbfir_ragged_tile_register(u, d, b, 0, 0, 0))
        base = RaggedPlan(sigs)
        outs = base.outputs
        base_ms = _time(base.run, reps)
        best, best_ms = None, base_ms
        for cand in ragged_candidates(u, d):
            _lib.check(lib.gbfir_ragged_tile_register(u, d, b, *cand))
            try:
                plan = RaggedPlan(sigs, outputs=outs)
                ms = _time(plan.run, reps)
            except _lib.GbfirError:
                continue
            if ms < best_ms:
                best, best_ms = cand, ms
        if best is None:
            _lib.check(lib.gbfir_ragged_tile_register(u, d, b, 0, 0, 0))
        else:
            _lib.check(lib.gbfir_ragged_tile_register(u, d, b, *best))
        results[f"{u}/{d}|L<={b}"] = {"tile": list(best) if best else "heuristic", "ms": best_ms,
                                      "heuristic_ms": base_ms, "signals": len(sigs)}
    return results
