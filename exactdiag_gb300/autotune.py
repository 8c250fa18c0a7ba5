"""Autotuner of the fused Lanczos step's launch and work shape.

For a sector shape (L, Nh, Nd, real/complex) and vector dtype it times a few steps for each
candidate and keeps the fastest, in two stages:

1. the free-row kernel's compiled register variant x persistent grid size (ed_sector_set_launch)
   x rows per lane worked on together, and the variant whose gathers go through shared memory
   (ed_sector_set_step_shape) -- these change only how work maps onto threads and CTAs, never a
   result bit;
2. for the winner, the offsets of a segment chunk's window (32: a lane's two rows in two segments;
   64: in one segment) x the rows of a segment chunk (the unit of work and of the step's partial
   sums): the sector is re-planned for each candidate, so its recursions' last bits follow the choice
   (the same for a sector alone and in a batch, which both apply it).

Results are cached as JSON keyed by GPU name and shape, so later runs apply the choice without
timing.  Cache file: $EXACTDIAG_GB300_AUTOTUNE, else ~/.cache/exactdiag_gb300/autotune.json.
"""

from __future__ import annotations

import ctypes
import json
import os
import pathlib

import numpy as np
import torch

from exactdiag_gb300 import _native as nat
from exactdiag_gb300.engine import DeviceSector

CANDIDATES = ((2, 0), (3, 0), (4, 0), (2, 1))  # (register variant: min resident CTAs per SM, CTAs per SM)
ROWS_PER_LANE = (1, 2)
# gathers through shared memory (cp.async): one compiled variant of 2 CTAs per SM, all that fit
STAGED_CANDIDATES = ((2, 0, 1), (2, 0, 2))  # (register variant, CTAs per SM, rows per lane)
CHUNK_ROWS = (2048, 4096, 8192, 16384, 32768)
DEFAULT_CHUNK_ROWS = 16384
WINDOWS = (32, 64)  # offsets of a segment chunk's window (64: not with staged gathers)
DEFAULT_WINDOW = 32


def cache_path() -> pathlib.Path:
    env = os.environ.get("EXACTDIAG_GB300_AUTOTUNE")
    if env:
        return pathlib.Path(env)
    return pathlib.Path.home() / ".cache" / "exactdiag_gb300" / "autotune.json"


def _key(sector: DeviceSector, dtype: torch.dtype) -> str:
    k = sector.key
    name = torch.cuda.get_device_name(sector.device)
    kind = "real" if sector.is_real else "complex"
    return f"{name}|L{k.num_rungs}|Nh{k.num_holes}|Nd{k.num_down_spins}|{kind}|{str(dtype).replace('torch.', '')}"


def _load() -> dict:
    p = cache_path()
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def _save(cache: dict) -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(".tmp")
        tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
        os.replace(tmp, p)
    except OSError:
        pass  # a read-only home is not an error: the choice is still applied for this process


def set_launch(sector: DeviceSector, min_ctas: int, ctas: int) -> None:
    nat.check("ed_sector_set_launch", sector._lib.ed_sector_set_launch(sector.handle, int(min_ctas), int(ctas)))


def set_step_shape(sector: DeviceSector, rows_per_lane: int, chunk_rows: int, staged: int = 0) -> None:
    nat.check("ed_sector_set_step_shape",
              sector._lib.ed_sector_set_step_shape(sector.handle, int(rows_per_lane), int(chunk_rows), int(staged)))


def get_step_shape(sector: DeviceSector) -> tuple[int, int, int]:
    a, c, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    nat.check("ed_sector_get_step_shape", sector._lib.ed_sector_get_step_shape(sector.handle, ctypes.byref(a),
                                                                               ctypes.byref(c), ctypes.byref(g)))
    return a.value, c.value, g.value


def set_window(sector: DeviceSector, offsets: int) -> None:
    nat.check("ed_sector_set_segment_window", sector._lib.ed_sector_set_segment_window(sector.handle, int(offsets)))


def get_window(sector: DeviceSector) -> int:
    w = ctypes.c_int()
    nat.check("ed_sector_get_segment_window", sector._lib.ed_sector_get_segment_window(sector.handle, ctypes.byref(w)))
    return w.value


def apply(sector: DeviceSector, rec: dict) -> None:
    """Set a tuned record's launch and work shape on a sector."""
    set_launch(sector, rec["min_ctas_per_sm"], rec["ctas_per_sm"])
    set_window(sector, DEFAULT_WINDOW)  # staged gathers need it; a 64-offset record is never staged
    set_step_shape(sector, rec.get("rows_per_lane", 0), rec.get("chunk_rows", DEFAULT_CHUNK_ROWS),
                   rec.get("staged", 0))
    set_window(sector, rec.get("window", DEFAULT_WINDOW))


def get_launch(sector: DeviceSector) -> tuple[int, int]:
    a, g = ctypes.c_int(), ctypes.c_int()
    nat.check("ed_sector_get_launch", sector._lib.ed_sector_get_launch(sector.handle, ctypes.byref(a),
                                                                       ctypes.byref(g)))
    return a.value, g.value


def row_kinds(sector: DeviceSector) -> tuple[int, int, int]:
    """Chunks of the fused step per row kind (free, stabiliser-resolved, orbit walk)."""
    c = (ctypes.c_int * 3)()
    nat.check("ed_sector_row_kinds", sector._lib.ed_sector_row_kinds(sector.handle, c))
    return int(c[0]), int(c[1]), int(c[2])


def kind_rows(sector: DeviceSector) -> tuple[int, int, int]:
    """Rows per row kind (free, stabiliser-resolved, orbit walk)."""
    c = (ctypes.c_int64 * 3)()
    nat.check("ed_sector_kind_rows", sector._lib.ed_sector_kind_rows(sector.handle, c))
    return int(c[0]), int(c[1]), int(c[2])


def step_launches(sector: DeviceSector) -> int:
    """Kernel launches of one ed_lanczos_step (ed_sector_step_launches): the expanded copies when
    the sector has any, one fused H.v kernel per row kind present, the scalar reduction, and the
    update (flat pass, exact-norm pass, exact b, scaling pass)."""
    c = ctypes.c_int()
    nat.check("ed_sector_step_launches", sector._lib.ed_sector_step_launches(sector.handle, ctypes.byref(c)))
    return int(c.value)


_MEMO: dict = {}
MIN_ROWS = 1 << 20  # smaller sectors keep the default launch: their steps take microseconds


def ensure(sector: DeviceSector, weights, dtype: torch.dtype) -> dict | None:
    """Apply the tuned launch for this sector shape and dtype: from this process's memo, else the
    JSON cache, else by timing the candidates once.  Sectors below MIN_ROWS rows, or with
    EXACTDIAG_GB300_NO_TUNE=1 set, keep the default launch (3 CTAs per SM, all that fit)."""
    if sector.n < MIN_ROWS or os.environ.get("EXACTDIAG_GB300_NO_TUNE") == "1":
        return None
    key = _key(sector, dtype)
    rec = _MEMO.get(key)
    if rec is None:
        rec = tune(sector, weights, dtype)
    else:
        apply(sector, rec)
    return rec


def tune(sector: DeviceSector, weights, dtype: torch.dtype, steps: int = 3, use_cache: bool = True) -> dict:
    """Apply the fastest launch configuration for this sector shape; returns the record used (also
    kept in this process's memo, which ensure() reads)."""
    rec = _tune(sector, weights, dtype, steps, use_cache)
    _MEMO[_key(sector, dtype)] = rec
    return rec


def _tune(sector: DeviceSector, weights, dtype: torch.dtype, steps: int, use_cache: bool) -> dict:
    key = _key(sector, dtype)
    cache = _load() if use_cache else {}
    if key in cache and "window" in cache[key]:
        rec = cache[key]
        apply(sector, rec)
        return dict(rec, cached=True)
    n = sector.n
    v = torch.as_tensor(np.random.default_rng(3).uniform(-1, 1, n), device=sector.device).to(dtype)
    buf = [v.clone(), torch.zeros_like(v)]
    scal = torch.zeros(2 * (steps + 2) + 4, dtype=torch.float64, device=sector.device)
    norm = torch.zeros(1, dtype=torch.float64, device=sector.device)
    sector.normalize(buf[0], norm)

    def time_steps() -> float:
        for k in range(steps + 1):
            if k == 1:
                torch.cuda.synchronize()
                start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                start.record()
            other = buf[(k + 1) % 2]
            sector.lanczos_step(weights, buf[k % 2], other if k else None, other, scal[2 * k: 2 * k + 4])
        stop.record()
        torch.cuda.synchronize()
        return start.elapsed_time(stop) / steps

    timings = {}
    set_window(sector, DEFAULT_WINDOW)
    set_step_shape(sector, 0, DEFAULT_CHUNK_ROWS)
    shapes = [(minb, ctas, nr, 0) for minb, ctas in CANDIDATES for nr in ROWS_PER_LANE]
    shapes += [(minb, ctas, nr, 1) for minb, ctas, nr in STAGED_CANDIDATES]
    for minb, ctas, nr, staged in shapes:
        try:
            set_launch(sector, minb, ctas)
            set_step_shape(sector, nr, DEFAULT_CHUNK_ROWS, staged)
        except nat.EngineError:
            continue
        timings[(minb, ctas, nr, staged, DEFAULT_WINDOW, DEFAULT_CHUNK_ROWS)] = time_steps()
    best = min(timings, key=timings.get)
    set_launch(sector, best[0], best[1])
    set_step_shape(sector, best[2], DEFAULT_CHUNK_ROWS, best[3])
    for win in WINDOWS:
        if win != DEFAULT_WINDOW and best[3]:
            continue  # staged gathers: 32-offset windows only
        set_window(sector, win)
        for rows in CHUNK_ROWS:
            if (win, rows) == (DEFAULT_WINDOW, DEFAULT_CHUNK_ROWS):
                continue
            set_step_shape(sector, best[2], rows, best[3])
            timings[(best[0], best[1], best[2], best[3], win, rows)] = time_steps()
        set_window(sector, DEFAULT_WINDOW)
    best = min(timings, key=timings.get)
    rec = {"min_ctas_per_sm": best[0], "ctas_per_sm": best[1], "rows_per_lane": best[2], "staged": best[3],
           "window": best[4], "chunk_rows": best[5], "ms_per_step": timings[best],
           "candidates": {",".join(str(v) for v in k): t for k, t in timings.items()},
           "candidate_key": "min_ctas_per_sm,ctas_per_sm,rows_per_lane,staged,window,chunk_rows"}
    apply(sector, rec)
    rec["grid"] = get_launch(sector)[1]
    cache[key] = rec
    if use_cache:
        _save(cache)
    return dict(rec, cached=False)
