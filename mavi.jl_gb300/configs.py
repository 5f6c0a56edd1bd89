"""Configuration objects mirroring Mavi.Configs (src/configs.jl).

Each class keeps the reference's field names and argument meaning; ``fill``
methods write them into the C structs of include/mavi_cuda.h.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Any, Sequence

from . import abi

# ---------------------------------------------------------------------------
# Geometries (src/configs.jl:28-229)
# ---------------------------------------------------------------------------


@dataclass
class RectangleCfg:
    """RectangleCfg(length, height, bottom_left) (src/configs.jl:34-51)."""
    length: float
    height: float
    bottom_left: tuple = (0.0, 0.0)

    @property
    def size(self):
        return (float(self.length), float(self.height))

    @staticmethod
    def from_points(points, offset=0.0) -> "RectangleCfg":
        """RectangleCfg(points; offset) (src/configs.jl:53-66)."""
        xs = [p[0] for p in points]
        ys = [p[1] for p in points]
        max_x, min_x = max(xs) + offset, min(xs) - offset
        max_y, min_y = max(ys) + offset, min(ys) - offset
        return RectangleCfg(length=max_x - min_x, height=max_y - min_y, bottom_left=(min_x, min_y))

    def fill(self, sp: abi.MaviSpace):
        sp.geometry = abi.MAVI_GEOM_RECTANGLE
        sp.length, sp.height = float(self.length), float(self.height)
        sp.bl_x, sp.bl_y = float(self.bottom_left[0]), float(self.bottom_left[1])

    def bounding_box(self) -> "RectangleCfg":
        return self


@dataclass
class CircleCfg:
    """CircleCfg(radius, center) (src/configs.jl:145-152)."""
    radius: float
    center: tuple = (0.0, 0.0)

    def fill(self, sp: abi.MaviSpace):
        sp.geometry = abi.MAVI_GEOM_CIRCLE
        sp.radius = float(self.radius)
        sp.cx, sp.cy = float(self.center[0]), float(self.center[1])

    def bounding_box(self) -> RectangleCfg:      # src/configs.jl:189-195
        r = float(self.radius)
        return RectangleCfg(2 * r, 2 * r, (self.center[0] - r, self.center[1] - r))


@dataclass
class LinesCfg:
    """LinesCfg(lines; bbox) (src/configs.jl:137-143): segments ((x1,y1),(x2,y2))."""
    lines: Sequence
    bbox: RectangleCfg | None = None

    def fill(self, sp: abi.MaviSpace):
        if not 1 <= len(self.lines) <= abi.MAVI_MAX_LINES:
            raise ValueError(f"LinesCfg supports 1..{abi.MAVI_MAX_LINES} lines")
        sp.geometry = abi.MAVI_GEOM_LINES
        sp.num_lines = len(self.lines)
        for k, (p1, p2) in enumerate(self.lines):
            sp.lines[k][0], sp.lines[k][1] = float(p1[0]), float(p1[1])
            sp.lines[k][2], sp.lines[k][3] = float(p2[0]), float(p2[1])
        if self.bbox is not None:
            sp.has_bbox = 1
            sp.bbox_length, sp.bbox_height = float(self.bbox.length), float(self.bbox.height)
            sp.bbox_bl_x, sp.bbox_bl_y = float(self.bbox.bottom_left[0]), float(self.bbox.bottom_left[1])

    def bounding_box(self) -> RectangleCfg:      # src/configs.jl:201-221
        if self.bbox is not None:
            return self.bbox
        xs = [c for (p1, p2) in self.lines for c in (p1[0], p2[0])]
        ys = [c for (p1, p2) in self.lines for c in (p1[1], p2[1])]
        return RectangleCfg(max(xs) - min(xs), max(ys) - min(ys), (min(xs), min(ys)))


# ---------------------------------------------------------------------------
# Wall types (src/configs.jl:235-279)
# ---------------------------------------------------------------------------


class RigidWalls:
    code = abi.MAVI_WALL_RIGID


class PeriodicWalls:
    code = abi.MAVI_WALL_PERIODIC


class SlipperyWalls:
    code = abi.MAVI_WALL_SLIPPERY


_MODES = {"outside": abi.MAVI_POTMODE_OUTSIDE, "inside": abi.MAVI_POTMODE_INSIDE,
          "repulsion": abi.MAVI_POTMODE_REPULSION}


@dataclass
class PotentialWalls:
    """PotentialWalls(potential, mode) (src/configs.jl:263-279)."""
    potential: Any
    mode: str = "repulsion"
    code = abi.MAVI_WALL_POTENTIAL

    def fill_potential(self, sp: abi.MaviSpace):
        sp.pot_mode = _MODES[self.mode]
        if isinstance(self.potential, HarmTruncCfg):
            sp.pot_kind = abi.MAVI_DYN_HARM_TRUNC
            p = self.potential
            vals = (p.k_rep, p.k_atr, p.dist_eq, p.dist_max)
        elif isinstance(self.potential, LenJonesCfg):
            sp.pot_kind = abi.MAVI_DYN_LEN_JONES
            vals = (self.potential.sigma, self.potential.epsilon, 0.0, 0.0)
        else:
            raise TypeError("PotentialWalls supports HarmTruncCfg and LenJonesCfg potentials")
        for k, v in enumerate(vals):
            sp.pot_params[k] = float(v)


@dataclass
class SpaceCfg:
    """SpaceCfg(wall_type, geometry_cfg) (src/configs.jl:285-302).

    ``SpaceCfg.many([(wall, geometry), ...])`` builds ManyWalls/ManyGeometries;
    the first entry is the main wall and geometry (src/configs.jl:304-312)."""
    wall_type: Any
    geometry_cfg: Any
    extra: list = field(default_factory=list)

    @staticmethod
    def many(entries) -> "SpaceCfg":
        entries = list(entries)
        if not 1 <= len(entries) <= abi.MAVI_MAX_SPACES:
            raise ValueError(f"SpaceCfg supports 1..{abi.MAVI_MAX_SPACES} (wall, geometry) entries")
        (w0, g0), rest = entries[0], entries[1:]
        return SpaceCfg(w0, g0, list(rest))

    @property
    def entries(self):
        return [(self.wall_type, self.geometry_cfg)] + list(self.extra)

    def fill(self, params: abi.MaviReplicaParams):
        ents = self.entries
        params.num_spaces = len(ents)
        for k, (w, g) in enumerate(ents):
            sp = params.spaces[k]
            g.fill(sp)
            sp.wall = w.code
            if isinstance(w, PotentialWalls):
                w.fill_potential(sp)

    def bounding_box(self) -> RectangleCfg:
        """get_bounding_box with the ManyGeometries fold (src/configs.jl:68-77, 223-229)."""
        bb = self.entries[0][1].bounding_box()
        for _, g in self.entries[1:]:
            b2 = g.bounding_box()
            max_x = max(bb.bottom_left[0] + bb.length, b2.bottom_left[0] + b2.length)
            max_y = max(bb.bottom_left[1] + bb.height, b2.bottom_left[1] + b2.height)
            min_x = min(bb.bottom_left[0], b2.bottom_left[0])
            min_y = min(bb.bottom_left[1], b2.bottom_left[1])
            bb = RectangleCfg(max_x - min_x, max_y - min_y, (min_x, min_y))
        return bb


# ---------------------------------------------------------------------------
# Dynamic configurations (src/configs.jl:318-421)
# ---------------------------------------------------------------------------


@dataclass
class HarmTruncCfg:
    """Truncated harmonic potential (src/configs.jl:341-368)."""
    k_rep: float
    k_atr: float
    dist_eq: float
    dist_max: float
    mobility: float = 1.0   # used by OverdampedStep only

    def fill(self, d: abi.MaviDynamicCfg):
        d.kind = abi.MAVI_DYN_HARM_TRUNC
        d.k_rep, d.k_atr, d.dist_eq, d.dist_max = map(float, (self.k_rep, self.k_atr, self.dist_eq, self.dist_max))
        d.mobility = float(self.mobility)


@dataclass
class LenJonesCfg:
    """Lennard-Jones potential, no cutoff (src/configs.jl:380-397)."""
    sigma: float
    epsilon: float
    mobility: float = 1.0

    def fill(self, d: abi.MaviDynamicCfg):
        d.kind = abi.MAVI_DYN_LEN_JONES
        d.sigma, d.epsilon = float(self.sigma), float(self.epsilon)
        d.mobility = float(self.mobility)


@dataclass
class SzaboCfg:
    """Szabo self-propelled model (src/configs.jl:399-408)."""
    vo: float
    mobility: float
    relax_time: float
    k_rep: float
    k_adh: float
    r_eq: float
    r_max: float
    rot_diff: float

    def fill(self, d: abi.MaviDynamicCfg):
        d.kind = abi.MAVI_DYN_SZABO
        for f in ("vo", "mobility", "relax_time", "k_rep", "k_adh", "r_eq", "r_max", "rot_diff"):
            setattr(d, f, float(getattr(self, f)))


@dataclass
class RunTumbleCfg:
    """Run-and-tumble particles with WCA repulsion (src/configs.jl:410-415)."""
    vo: float
    sigma: float
    epsilon: float
    tumble_rate: float

    def fill(self, d: abi.MaviDynamicCfg):
        d.kind = abi.MAVI_DYN_RUN_TUMBLE
        for f in ("vo", "sigma", "epsilon", "tumble_rate"):
            setattr(d, f, float(getattr(self, f)))


def particle_radius(cfg) -> float:
    """particle_radius (src/configs.jl:418-421)."""
    if isinstance(cfg, (LenJonesCfg, RunTumbleCfg)):
        return cfg.sigma * 2 ** (1 / 6) / 2
    if isinstance(cfg, SzaboCfg):
        return cfg.r_eq / 2
    if isinstance(cfg, HarmTruncCfg):
        return cfg.dist_eq / 2.0
    if hasattr(cfg, "particle_radius"):
        return cfg.particle_radius()
    raise TypeError(f"no particle radius for {type(cfg).__name__}")


# ---------------------------------------------------------------------------
# Integration configuration (src/configs.jl:469-490)
# ---------------------------------------------------------------------------


@dataclass
class ChunksCfg:
    """ChunksCfg(num_cols, num_rows) (src/configs.jl:477-480)."""
    num_cols: int
    num_rows: int


@dataclass
class CUDADevice:
    """The GPU device mode: the counterpart of the reference's DeviceMode
    (Sequencial / Threaded, src/configs.jl:471-475) that routes the step loop
    to libmavi_cuda.so.

    precision: "fp64" (every operation in double; the drop-in) or "mixed"
    (FP32 pair loop on chunk-centre offsets, FP64 update, wrap and binning).
    noise: "device" (Philox on the GPU, seeded) or "injected" (the caller
    supplies each step's noise numbers).
    gather: pair gather — "staged" (warp window in shared memory), "global"
    (chunk by chunk), "columns" (contiguous row ranges per column), which give
    identical results; for the mixed Lennard-Jones / WCA passes also "tiles"
    (Newton's third law inside tiles of chunks, a CTA per tile) and
    "tiles_queue" (the same tiles pulled from a device work queue by
    persistent CTAs), identical to each other; for the mixed
    harmonic-truncated and Szabo passes also "lanes2" / "lanes4" (the column
    gather with 2 or 4 lanes per particle, partial sums combined in a fixed
    order); for the mixed Lennard-Jones passes also "split" (pairs at
    r >= 2 sigma in plain FP32, closer ones in double-float); or "auto"
    (the fastest force pass at creation).
    tune_cache: a JSON file (or the MAVI_TUNE_CACHE environment variable) in
    which "auto" records its choice per workload shape; later handles of
    the same shape take the recorded mode without timing (tuning.py)."""
    precision: str = "fp64"
    device: int = 0
    use_graph: bool = True
    noise: str = "device"
    seed: int = 0
    gather: str = "auto"
    tune_cache: str | None = None

    def options(self) -> abi.MaviOptions:
        o = abi.MaviOptions()
        o.precision = {"fp64": abi.MAVI_PREC_FP64, "mixed": abi.MAVI_PREC_MIXED}[self.precision]
        o.noise_mode = {"device": abi.MAVI_NOISE_DEVICE, "injected": abi.MAVI_NOISE_INJECTED}[self.noise]
        o.seed = int(self.seed) & ((1 << 64) - 1)
        o.device = int(self.device)
        o.use_graph = 1 if self.use_graph else 0
        o.gather_mode = {"auto": -1, "staged": 0, "global": 1, "columns": 2, "tiles": 3, "tiles_queue": 4,
                         "lanes2": 5, "lanes4": 6, "split": 7}[self.gather]
        return o


@dataclass
class IntCfg:
    """IntCfg(dt, chunks_cfg, device, extra) (src/configs.jl:482-487)."""
    dt: float
    chunks_cfg: ChunksCfg | None = None
    device: CUDADevice = field(default_factory=CUDADevice)
    extra: Any = None


def has_chunks(int_cfg: IntCfg) -> bool:
    return int_cfg.chunks_cfg is not None


def chunk_capacity(chunk_length: float, chunk_height: float, particle_r: float) -> int:
    """Chunk capacity (src/chunks.jl:32-34)."""
    nc = (math.ceil(0.5 * chunk_length / particle_r) + 1) * (math.ceil(0.5 * chunk_height / particle_r) + 1)
    return int(math.ceil(nc * 2))
