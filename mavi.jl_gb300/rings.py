"""The rings model mirroring Mavi.Rings (src/rings/*.jl): ring polymers of
particles with pair excluded volume, springs, an area term, self-propulsion
along a per-ring polarisation, plus an optional bending term (``k_bend``;
zero reproduces the reference, which has none)."""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Any, Sequence

import numpy as np

from . import abi
from .configs import HarmTruncCfg, IntCfg, ChunksCfg, CUDADevice, CircleCfg, RectangleCfg, chunk_capacity
from .system import System, TimeInfo


# ---------------------------------------------------------------------------
# configs (src/rings/configs.jl)
# ---------------------------------------------------------------------------
@dataclass
class InteractionMatrix:
    """InteractionMatrix (src/rings/configs.jl:292-316): HarmTruncCfg per pair of types."""
    matrix: Sequence[Sequence[HarmTruncCfg]]

    def get(self, t1: int, t2: int) -> HarmTruncCfg:     # 1-based types
        return self.matrix[t1 - 1][t2 - 1]

    @property
    def num_types(self) -> int:
        return len(self.matrix)


def _per_type(v, n):
    if isinstance(v, (list, tuple, np.ndarray)):
        if len(v) != n:
            raise ValueError("per-type parameter has the wrong length")
        return [float(x) for x in v]
    return [float(v)] * n


@dataclass
class RingsCfg:
    """RingsCfg (src/rings/configs.jl:326-381). Scalars or one value per type."""
    p0: Any
    relax_time: Any
    vo: Any
    mobility: Any
    rot_diff: Any
    k_area: Any
    k_spring: Any
    l_spring: Any
    interaction_finder: Any
    num_particles: Any = -1
    k_bend: Any = 0.0

    @property
    def num_types(self) -> int:
        if isinstance(self.interaction_finder, InteractionMatrix):
            return self.interaction_finder.num_types
        lens = [len(v) for v in (self.p0, self.relax_time, self.vo, self.mobility, self.rot_diff, self.k_area,
                                 self.k_spring, self.l_spring) if isinstance(v, (list, tuple, np.ndarray))]
        return max(lens) if lens else 1

    def interaction(self, t1: int, t2: int) -> HarmTruncCfg:
        f = self.interaction_finder
        return f.get(t1, t2) if isinstance(f, InteractionMatrix) else f

    def type_value(self, name: str, t: int) -> float:     # 1-based
        return _per_type(getattr(self, name), self.num_types)[t - 1]

    def particle_radius(self):
        """Minimum particle radius over types (src/rings/configs.jl:438-443)."""
        return min(self.interaction(t, t).dist_eq / 2.0 for t in range(1, self.num_types + 1))

    def ring_num_particles(self, t: int = 1) -> int:
        n = self.num_particles
        return int(n[t - 1]) if isinstance(n, (list, tuple, np.ndarray)) else int(n)

    def fill(self, d: abi.MaviDynamicCfg):
        d.kind = abi.MAVI_DYN_RINGS

    def fill_rings(self, rc: abi.MaviRingsCfg, num_rings: int, nmax: int, num_particles):
        nt = self.num_types
        if nt > abi.MAVI_MAX_TYPES:
            raise ValueError(f"at most {abi.MAVI_MAX_TYPES} ring types")
        rc.num_types, rc.num_rings, rc.nmax = nt, num_rings, nmax
        nps = num_particles if isinstance(num_particles, (list, tuple, np.ndarray)) else [num_particles] * nt
        for t in range(nt):
            rc.num_particles[t] = int(nps[t])
            for name in ("p0", "relax_time", "vo", "mobility", "rot_diff", "k_area", "k_spring", "l_spring", "k_bend"):
                getattr(rc, name)[t] = self.type_value(name, t + 1)
            for u in range(nt):
                it = self.interaction(t + 1, u + 1)
                rc.inter_k_rep[t][u] = float(it.k_rep)
                rc.inter_k_atr[t][u] = float(it.k_atr)
                rc.inter_dist_eq[t][u] = float(it.dist_eq)
                rc.inter_dist_max[t][u] = float(it.dist_max)


def get_area0(cfg: RingsCfg, t: int = 1) -> float:
    """get_area0 (src/rings/configs.jl:452-457)."""
    n = cfg.ring_num_particles(t)
    return (n * cfg.type_value("l_spring", t) / cfg.type_value("p0", t)) ** 2


def get_equilibrium_p0(num_particles: int) -> float:
    """get_equilibrium_p0 (src/rings/configs.jl:464-468)."""
    theta = 2 * math.pi / num_particles
    return 2 * (num_particles * (1 - math.cos(theta)) / math.sin(theta)) ** .5


def get_ring_radius(p_radius: float, num_particles: int) -> float:
    """get_ring_radius (src/rings/utils.jl:5-7): radius of the polygon whose
    consecutive vertices are 2*p_radius apart."""
    return (p_radius * 2) / (2 * (1 - math.cos(2 * math.pi / num_particles))) ** .5


@dataclass
class InvasionsCfg:
    """InvasionsCfg(steps_to_update) (src/rings/configs.jl:334-336)."""
    steps_to_update: int


@dataclass
class IntCfgExtra:
    """IntCfgExtra(r_chunks_cfg, invasions_cfg) (src/rings/configs.jl:338-341)."""
    r_chunks_cfg: ChunksCfg | None = None
    invasions_cfg: InvasionsCfg | None = None


def RingsIntCfg(dt: float, p_chunks_cfg: ChunksCfg | None = None, r_chunks_cfg: ChunksCfg | None = None,
                invasions_cfg: InvasionsCfg | None = None, device: CUDADevice | None = None) -> IntCfg:
    """RingsIntCfg (src/rings/configs.jl:344-350)."""
    return IntCfg(dt=dt, chunks_cfg=p_chunks_cfg, device=device or CUDADevice(),
                  extra=IntCfgExtra(r_chunks_cfg, invasions_cfg))


@dataclass(frozen=True)
class Invasion:
    """Invasion (src/rings/rings.jl:89-93): particle p_id (1-based scalar
    index) of ring invasor (1-based) inside ring invaded."""
    invasor: int
    invaded: int
    p_id: int


@dataclass
class InvasionsInfo:
    """InvasionsInfo(list, last_check) (src/rings/rings.jl:95-100)."""
    list: list
    last_check: int


# ---------------------------------------------------------------------------
# state (src/rings/states.jl)
# ---------------------------------------------------------------------------
class RingsState:
    """RingsState (src/rings/states.jl:74-124). ``rings_pos`` has shape
    (num_rings, nmax, 2): the bytes of Julia's column-major
    Matrix{SVector{2}}(nmax, num_rings); ``pos`` is the flat (num_rings*nmax, 2)
    view sharing memory with it. ``types`` are 1-based per ring (or None)."""
    kind = abi.MAVI_STATE_RINGS

    def __init__(self, rings_pos, pol, num_particles=None, types=None, active_state=None):
        rp = np.ascontiguousarray(np.asarray(rings_pos, dtype=np.float64))
        if rp.ndim != 3 or rp.shape[2] != 2:
            raise ValueError("rings_pos must have shape (num_rings, nmax, 2)")
        self.rings_pos = rp
        self.pos = rp.reshape(-1, 2)
        self.pol = np.ascontiguousarray(np.asarray(pol, dtype=np.float64).reshape(-1))
        self.num_rings, self.nmax = rp.shape[0], rp.shape[1]
        if self.pol.shape[0] != self.num_rings:
            raise ValueError("pol must have one entry per ring")
        self.num_particles = self.nmax if num_particles is None else num_particles
        self.types = None if types is None else np.ascontiguousarray(np.asarray(types, dtype=np.int32))
        self.vel = None
        self.active_state = active_state

    def types_array(self):
        return self.types if self.types is not None else np.ones(self.num_rings, dtype=np.int32)

    def pol_array(self):
        return self.pol

    def ring_num_particles(self, ring: int) -> int:
        n = self.num_particles
        if isinstance(n, (list, tuple, np.ndarray)):
            return int(n[self.types_array()[ring] - 1])
        return int(n)


@dataclass
class NeighborsCfg:
    """NeighborsCfg(only_count, type, tol) (src/rings/neighbors.jl:10-14) for the
    particle neighbour lists; type "rings" ignores particles of the same ring,
    "all" counts every particle."""
    only_count: bool = False
    type: str = "all"
    tol: float = 1.1


# ---------------------------------------------------------------------------
# variable number of rings: ActiveState, sources and sinks
# (src/states.jl:14-20, src/rings/states.jl:20-40, src/rings/sources.jl)
# ---------------------------------------------------------------------------
class ActiveState:
    """ActiveState(mask) (src/states.jl:14-20): which rings are active at the
    start; a bool applies to every ring."""

    def __init__(self, mask=True):
        self.mask = mask

    def get_active_mask(self, num_rings: int) -> np.ndarray:
        if isinstance(self.mask, (bool, np.bool_)):
            return np.full(num_rings, bool(self.mask))
        m = np.asarray(self.mask, dtype=bool).reshape(-1)
        if m.size != num_rings:
            raise ValueError("the active mask needs one entry per ring")
        return m


@dataclass
class SourceCfg:
    """SourceCfg (src/rings/sources.jl:27-48): a ring spawn template
    (``spawn_pos``, nmax points) repeated on a size[0] x size[1] grid of boxes
    from ``bottom_left``; a ring is added to every box that holds no particle
    (within ``pad``). ``spawn_pol`` is an angle or "random"."""
    bottom_left: tuple
    spawn_pos: object
    spawn_pol: object = 0.0
    pad: float = 0.0
    offset: tuple = (0.0, 0.0)
    size: tuple = (1, 1)


@dataclass
class SinkCfg:
    """SinkCfg (src/rings/sources.jl:241-244): rings whose centre of mass lies
    in ``geometry_cfg`` (RectangleCfg or CircleCfg) are removed."""
    geometry_cfg: object


def _rect_union(a, b):
    """RectangleCfg + RectangleCfg (src/configs.jl:68-77): (bl_x, bl_y, length, height)."""
    max_x = max(a[0] + a[2], b[0] + b[2])
    max_y = max(a[1] + a[3], b[1] + b[3])
    min_x = min(a[0], b[0])
    min_y = min(a[1], b[1])
    return (min_x, min_y, max_x - min_x, max_y - min_y)


def _intersects(r1, r2):
    """check_intersection(r1, r2) of two rectangles (src/configs.jl:79-87),
    (bl_x, bl_y, length, height) each."""
    x1 = r2[0] <= r1[0] <= r2[0] + r2[2]
    x2 = r2[0] <= r1[0] + r1[2] <= r2[0] + r2[2]
    y1 = r2[1] <= r1[1] <= r2[1] + r2[3]
    y2 = r2[1] <= r1[1] + r1[3] <= r2[1] + r2[3]
    return (x1 or x2) and (y1 or y2)


def source_boxes(cfg: SourceCfg, chunk_grid=None):
    """The fields of Source(cfg, ...) (src/rings/sources.jl:122-185), in FP64
    with the reference's operation order: the spawn boxes (bl_x, bl_y, length,
    height), their spawn points and, with a chunk grid (bl_x, bl_y, length,
    height, rows, cols), the ChunksChecker's chunk lists ((row, col), 0-based);
    without one, None (PosChecker)."""
    sp = np.asarray(cfg.spawn_pos, dtype=np.float64).reshape(-1, 2)
    pad = float(cfg.pad)
    min_x, max_x = float(sp[:, 0].min()), float(sp[:, 0].max())
    min_y, max_y = float(sp[:, 1].min()), float(sp[:, 1].max())
    bbox_length = max_x - min_x + 2 * pad
    bbox_height = max_y - min_y + 2 * pad
    blx, bly = float(cfg.bottom_left[0]), float(cfg.bottom_left[1])
    ox, oy = float(cfg.offset[0]), float(cfg.offset[1])
    boxes, pads = [], []
    for i in range(1, int(cfg.size[0]) + 1):
        for j in range(1, int(cfg.size[1]) + 1):
            bx = blx + ((i - 1) * bbox_length + i * ox)
            by = bly + ((j - 1) * bbox_height + j * oy)
            boxes.append((bx, by, bbox_length, bbox_height))
            pads.append((bx - pad, by - pad, bbox_length + 2 * pad, bbox_height + 2 * pad))
    spawns = []
    for b in boxes:
        dx = b[0] - min_x + pad
        dy = b[1] - min_y + pad
        spawns.append(np.stack([sp[:, 0] + dx, sp[:, 1] + dy], axis=1))
    if chunk_grid is None:
        return boxes, spawns, None
    gblx, gbly, glen, ghei, rows, cols = chunk_grid
    cl, ch = glen / cols, ghei / rows
    glob = pads[0]
    for r in pads[1:]:
        glob = _rect_union(glob, r)
    tlx, tly = gblx + 0.0, gbly + ghei
    found, sx, ex = False, 0, 0
    for i in range(1, cols + 1):
        x1 = tlx + (i - 1) * cl
        x2 = x1 + cl
        if not found and x1 <= glob[0] <= x2:
            found, sx = True, i
        if found and x1 >= glob[0] + glob[2]:
            ex = i - 1
            break
    found, sy, ey = False, 0, 0
    for i in range(1, rows + 1):
        y2 = tly - (i - 1) * ch
        y1 = y2 - ch
        if not found and y1 <= glob[1] + glob[3] <= y2:
            found, sy = True, i
        if found and y2 <= glob[1]:
            ey = i - 1
            break
    lists = [[] for _ in pads]
    for col in range(sx, ex + 1):
        for row in range(sy, ey + 1):
            rect = (tlx + (col - 1) * cl, tly - row * ch, cl, ch)   # get_chunk_rect (src/chunks.jl:50-59)
            for k, bp in enumerate(pads):
                if _intersects(rect, bp):
                    lists[k].append((row - 1, col - 1))
    return boxes, spawns, lists


class RingsSystem(System):
    """RingsSystem (src/rings/rings.jl:231-291) on the GPU. With
    ``p_neighbors_cfg`` every pair pass also records the particle neighbour
    lists (``neighbors()``)."""
    is_rings = True

    def __init__(self, state: RingsState, space_cfg, dynamic_cfg: RingsCfg, int_cfg: IntCfg,
                 time_info: TimeInfo | None = None, p_neighbors_cfg: NeighborsCfg | None = None,
                 source_cfg=None):
        super().__init__(state, space_cfg, dynamic_cfg, int_cfg, time_info)
        if dynamic_cfg.num_types > 1 and state.types is None:
            raise ValueError("DynamicCfg has multiple types, but state.types is nothing!")
        self.p_neighbors_cfg = p_neighbors_cfg
        if source_cfg is not None and not isinstance(source_cfg, (list, tuple)):
            source_cfg = [source_cfg]
        self.source_cfg = None if source_cfg is None else list(source_cfg)
        for c in self.source_cfg or []:
            if not isinstance(c, (SourceCfg, SinkCfg)):
                raise ValueError(f"Unknown source configuration type: {type(c).__name__}")
            if isinstance(c, SourceCfg) and np.asarray(c.spawn_pos).reshape(-1, 2).shape[0] != state.nmax:
                raise ValueError("spawn_pos needs one point per row of rings_pos (nmax)")

    @property
    def variable_rings(self) -> bool:
        """VarRingsIds: an ActiveState was given or sources/sinks are configured."""
        return self.source_cfg is not None or getattr(self.state, "active_state", None) is not None

    def sources_abi(self):
        """(active_mask, entries, boxes, spawn_xy, chunk_rc) for
        mavi_rings_sources, or None without variable rings."""
        if not self.variable_rings:
            return None
        st = self.state
        a = getattr(st, "active_state", None)
        mask = (a.get_active_mask(st.num_rings) if a is not None else np.ones(st.num_rings, bool)).astype(np.int32)
        grid = None
        cc = self.int_cfg.chunks_cfg
        if cc is not None:
            bb = self.space_cfg.bounding_box()
            grid = (float(bb.bottom_left[0]), float(bb.bottom_left[1]), float(bb.length), float(bb.height),
                    int(cc.num_rows), int(cc.num_cols))
        cfgs = self.source_cfg or []
        entries = (abi.MaviSourceEntry * max(len(cfgs), 1))()
        boxes, spawn, chunks = [], [], []
        for k, c in enumerate(cfgs):
            e = entries[k]
            if isinstance(c, SinkCfg):
                e.kind = abi.MAVI_SRC_SINK
                g = c.geometry_cfg
                if isinstance(g, CircleCfg):
                    e.geometry = abi.MAVI_GEOM_CIRCLE
                    e.radius, e.cx, e.cy = float(g.radius), float(g.center[0]), float(g.center[1])
                elif isinstance(g, RectangleCfg):
                    e.geometry = abi.MAVI_GEOM_RECTANGLE
                    e.length, e.height = float(g.length), float(g.height)
                    e.bl_x, e.bl_y = float(g.bottom_left[0]), float(g.bottom_left[1])
                else:
                    raise ValueError("a sink geometry is a RectangleCfg or a CircleCfg")
                continue
            e.kind = abi.MAVI_SRC_SOURCE
            random_pol = isinstance(c.spawn_pol, str)
            if random_pol and c.spawn_pol != "random":
                raise ValueError("spawn_pol is an angle or 'random'")
            e.pol_mode = abi.MAVI_SPAWN_POL_RANDOM if random_pol else abi.MAVI_SPAWN_POL_FIXED
            e.pol = 0.0 if random_pol else float(c.spawn_pol)
            e.pad = float(c.pad)
            bx, sp, lists = source_boxes(c, grid)
            e.num_boxes = len(bx)
            for q, b in enumerate(bx):
                mb = abi.MaviSpawnBox()
                mb.bl_x, mb.bl_y, mb.length, mb.height = b
                mb.num_chunks = -1 if lists is None else len(lists[q])
                boxes.append(mb)
                spawn.append(sp[q])
                if lists is not None:
                    chunks.extend(lists[q])
        nb = len(boxes)
        box_arr = (abi.MaviSpawnBox * max(nb, 1))(*boxes)
        spawn_xy = np.ascontiguousarray(np.concatenate(spawn).reshape(-1)) if spawn else np.zeros(2)
        chunk_rc = np.ascontiguousarray(np.asarray(chunks, dtype=np.int32).reshape(-1)) if chunks else \
            np.zeros(2, dtype=np.int32)
        return mask, len(cfgs), entries, box_arr, spawn_xy, chunk_rc

    def invasions_abi(self):
        """(enable, steps_to_update, num_cols, num_rows) for
        mavi_rings_invasions_config, or None without an InvasionsCfg."""
        extra = getattr(self.int_cfg, "extra", None)
        inv = getattr(extra, "invasions_cfg", None)
        if inv is None:
            return None
        rc = getattr(extra, "r_chunks_cfg", None)
        return (1, int(inv.steps_to_update), int(rc.num_cols) if rc is not None else 0,
                int(rc.num_rows) if rc is not None else 0)

    def _configure_replica(self, h, replica: int):
        """Handle hook: variable rings ids and sources/sinks of this replica,
        then invasion detection (constructed last, as RingsSystem does)."""
        cfg = self.sources_abi()
        if cfg is not None:
            mask, n, entries, boxes, spawn_xy, chunk_rc = cfg
            h.check(h.lib.mavi_rings_sources(h.handle, replica, abi.as_iptr(mask), n, entries, boxes,
                                             abi.as_dptr(spawn_xy), abi.as_iptr(chunk_rc)), "mavi_rings_sources")
        inv = self.invasions_abi()
        if inv is not None:
            h.check(h.lib.mavi_rings_invasions_config(h.handle, replica, *inv), "mavi_rings_invasions_config")

    def invasions(self) -> InvasionsInfo:
        """RingsInfo.invasions: the list of the last check (every check's,
        appended, without ring chunks) and last_check."""
        h, k = self._replica()
        n, last = C.c_int64(), C.c_int64()
        h.check(h.lib.mavi_rings_invasions(h.handle, k, None, 0, C.byref(n), C.byref(last)), "mavi_rings_invasions")
        out = (abi.MaviInvasion * max(n.value, 1))()
        h.check(h.lib.mavi_rings_invasions(h.handle, k, out, n.value, C.byref(n), C.byref(last)),
                "mavi_rings_invasions")
        return InvasionsInfo([Invasion(out[q].invasor, out[q].invaded, out[q].p_id) for q in range(n.value)],
                             int(last.value))

    def _replica(self):
        """(handle, replica index) of this system: its own handle, or the
        SystemBatch's that drives it."""
        b = getattr(self, "_batch", None)
        if b is not None:
            return b.handle, b.handle.systems.index(self)
        return self._ensure(), 0

    def areas(self) -> np.ndarray:
        """RingsInfo.areas (src/rings/integration.jl:140-160): ring areas at
        the last force evaluation."""
        h, k = self._replica()
        out = np.zeros(self.state.num_rings)
        h.check(h.lib.mavi_rings_areas(h.handle, k, abi.as_dptr(out)), "mavi_rings_areas")
        return out

    def rings_ids(self):
        """(active_mask[num_rings] bool, uids[num_rings], num_active) on the
        device (VarRingsIds: mask, uids, num_active)."""
        h, k = self._replica()
        nr = self.state.num_rings
        mask = np.zeros(nr, dtype=np.int32)
        uids = np.zeros(nr, dtype=np.int32)
        na = C.c_int32()
        h.check(h.lib.mavi_rings_active(h.handle, k, abi.as_iptr(mask), abi.as_iptr(uids), C.byref(na)),
                "mavi_rings_active")
        return mask.astype(bool), uids, int(na.value)

    def _ensure(self, step_kind=None):
        fresh = self._handle is None
        h = super()._ensure(step_kind)
        if self.p_neighbors_cfg is not None and (fresh or h is not getattr(self, "_nb_handle", None)):
            c = self.p_neighbors_cfg
            h.check(h.lib.mavi_rings_neighbors_config(h.handle, 1, 1 if c.only_count else 0,
                                                      1 if c.type == "all" else 0, float(c.tol)),
                    "mavi_rings_neighbors_config")
            self._nb_handle = h
        return h

    def neighbors(self):
        """(counts[num_slots], lists[num_slots, 15] or None): the particle
        neighbour lists at the last pair pass, 0-based slot ids, -1 padded."""
        if self.p_neighbors_cfg is None:
            raise RuntimeError("p_neighbors_cfg was not given")
        h = self._ensure()
        n = self.num_slots
        counts = np.zeros(n, dtype=np.int32)
        lists = None if self.p_neighbors_cfg.only_count else np.zeros(n * abi.MAVI_MAX_NEIGHBORS, dtype=np.int32)
        h.check(h.lib.mavi_rings_neighbors(h.handle, 0, abi.as_iptr(counts), abi.as_iptr(lists)),
                "mavi_rings_neighbors")
        return counts, (None if lists is None else lists.reshape(n, abi.MAVI_MAX_NEIGHBORS))

    @property
    def num_slots(self) -> int:
        return self.state.num_rings * self.state.nmax

    @property
    def num_pol(self) -> int:
        return self.state.num_rings

    def fill_params(self, p: abi.MaviReplicaParams, step_kind: int):
        super().fill_params(p, step_kind)
        nps = self.state.num_particles
        if isinstance(self.dynamic_cfg.num_particles, (list, tuple, np.ndarray)) or self.dynamic_cfg.num_particles != -1:
            nps = self.dynamic_cfg.num_particles
        self.dynamic_cfg.fill_rings(p.rings, self.state.num_rings, self.state.nmax, nps)

    def chunk_capacity(self) -> int:
        bb = self.space_cfg.bounding_box()
        cc = self.int_cfg.chunks_cfg
        return chunk_capacity(bb.length / cc.num_cols, bb.height / cc.num_rows, self.dynamic_cfg.particle_radius())


# ---------------------------------------------------------------------------
# initial states (src/rings/init_states.jl)
# ---------------------------------------------------------------------------
def create_circle(center, radius: float, num_p: int) -> np.ndarray:
    """create_circle (src/rings/init_states.jl:10-25): (num_p, 2) points."""
    theta = 2 * math.pi / num_p
    out = np.empty((num_p, 2))
    for i in range(num_p):
        out[i, 0] = radius * math.cos(i * theta) + center[0]
        out[i, 1] = radius * math.sin(i * theta) + center[1]
    return out


def rectangular_grid(num_cols: int, num_rows: int, num_particles, p_radius, types=None,
                     pad_x: float = 0.0, pad_y: float = 0.0, radius_k: float = 1.0):
    """Rings on a rectangular grid (src/rings/init_states.jl:27-72).
    Returns (rings_pos (num_rings, nmax, 2), RectangleCfg)."""
    from .configs import RectangleCfg
    if types is None:
        num_particles = [num_particles]
        p_radius = [p_radius]
        types = [1] * (num_cols * num_rows)
    ring_r = [get_ring_radius(pr, n) for pr, n in zip(p_radius, num_particles)]
    ring_length = [2 * (r + pr) for r, pr in zip(ring_r, p_radius)]
    max_ring_r, max_ring_length, nmax = max(ring_r), max(ring_length), max(num_particles)
    pad_x = pad_x * max_ring_r
    pad_y = pad_y * max_ring_r
    rp = np.zeros((num_cols * num_rows, nmax, 2))
    idx = 0
    for col in range(num_cols):
        for row in range(num_rows):
            cx = pad_x / 2 + col * (max_ring_length + pad_x) + max_ring_length / 2
            # the reference spaces rows with pad_x as well
            cy = pad_y / 2 + row * (max_ring_length + pad_x) + max_ring_length / 2
            t = types[idx]
            n = num_particles[t - 1]
            rp[idx, :n] = create_circle((cx, cy), ring_r[t - 1] * radius_k, n)
            idx += 1
    geom = RectangleCfg(length=num_cols * (pad_x + max_ring_length), height=num_rows * (pad_y + max_ring_length))
    return rp, geom


def random_pol(num_rings: int, rng=None) -> np.ndarray:
    """random_pol (src/rings/init_states.jl:74-80)."""
    rng = rng or np.random.default_rng()
    return rng.random(num_rings) * 2 * math.pi
