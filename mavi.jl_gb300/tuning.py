"""A JSON cache of the pair-pass autotuner's choices, keyed by workload shape.

With ``gather = "auto"`` (the default) ``mavi_create`` times the pair passes
and keeps the fastest (a mode that changes the bits must win by 10 %). That
timing costs a few force passes per handle, and on a busy device two handles
of one workload could in principle choose differently. With a cache file
(``CUDADevice(tune_cache=path)``, or the ``MAVI_TUNE_CACHE`` environment
variable), the first handle of a workload shape records its choice there and
later handles of the same shape are created with that mode directly: no
timing, and the same bits every time. The shape is what the choice depends
on — the dynamic, the precision, the step, the number of replicas, the total
particle count and the mean chunk occupancy (the last three in half-octave
buckets), and whether the replicas are periodic or have chunk grids.

The reference has no counterpart (its `Threaded` mode has nothing to tune);
the tuned quantity is how the pair loop over the chunk grid of
src/chunks.jl:26-40 / src/configs.jl:477-480 is laid out on the GPU.
"""
from __future__ import annotations

import json
import math
import os
import pathlib
import tempfile

from . import abi

_NAMES = {0: "staged", 1: "global", 2: "columns", 3: "tiles", 4: "tiles_queue", 5: "lanes2", 6: "lanes4",
          7: "split"}
VERSION = 1


def _bucket(x: float) -> float:
    """Half-octave bucket of a positive quantity (0 stays 0)."""
    return 0.0 if x <= 0 else round(2.0 * math.log2(x)) / 2.0


def shape_key(systems, step_kind: int, precision: str) -> str:
    """The workload-shape key of a handle over `systems`."""
    s0 = systems[0]
    n = sum(int(s.num_slots) for s in systems)
    chunks = 0
    gridless = False
    periodic = False
    for s in systems:
        cc = getattr(s.int_cfg, "chunks_cfg", None)
        if cc is None:
            gridless = True
        else:
            chunks += int(cc.num_rows) * int(cc.num_cols)
        periodic = periodic or type(s.space_cfg.wall_type).__name__ == "PeriodicWalls"
    occupancy = n / chunks if chunks else 0.0
    parts = [type(s0.dynamic_cfg).__name__, precision, f"step{int(step_kind)}", f"R{_bucket(len(systems))}",
             f"N{_bucket(n)}", f"occ{_bucket(occupancy)}", "gridless" if gridless else "grid",
             "periodic" if periodic else "open"]
    return "/".join(parts)


class TuneCache:
    """The cache file: {"version": 1, "entries": {shape key: {"gather_mode": m, "gather": name}}}."""

    def __init__(self, path):
        self.path = pathlib.Path(path)

    def _load(self) -> dict:
        try:
            d = json.loads(self.path.read_text())
            if d.get("version") == VERSION and isinstance(d.get("entries"), dict):
                return d
        except (OSError, ValueError):
            pass
        return {"version": VERSION, "entries": {}}

    def get(self, key: str):
        e = self._load()["entries"].get(key)
        m = e.get("gather_mode") if isinstance(e, dict) else None
        return int(m) if isinstance(m, int) and m in _NAMES else None

    def put(self, key: str, mode: int) -> None:
        d = self._load()
        d["entries"][key] = {"gather_mode": int(mode), "gather": _NAMES.get(int(mode), "?")}
        self.path.parent.mkdir(parents=True, exist_ok=True)
        # write to a temporary file beside it, then rename: readers never see a half file
        fd, tmp = tempfile.mkstemp(dir=str(self.path.parent), prefix=self.path.name, suffix=".tmp")
        with os.fdopen(fd, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def cache_for(device) -> TuneCache | None:
    """The cache a device configuration asks for, or None."""
    path = getattr(device, "tune_cache", None) or os.environ.get("MAVI_TUNE_CACHE")
    return TuneCache(path) if path else None


def tuned_options(systems, step_kind: int, device) -> tuple:
    """MaviOptions for a new handle, with the cached mode when the gather is
    autotuned and the cache holds this shape; returns (options, cache, key),
    cache/key not None when the handle's choice is to be recorded."""
    opt = device.options()
    cache = cache_for(device)
    if cache is None or opt.gather_mode >= 0:
        return opt, None, None
    key = shape_key(systems, step_kind, device.precision)
    mode = cache.get(key)
    if mode is not None:
        opt.gather_mode = mode
        return opt, None, None
    return opt, cache, key


def record(cache: TuneCache | None, key: str | None, stats: abi.MaviStats) -> None:
    if cache is not None and key is not None:
        cache.put(key, int(stats.gather_mode))
