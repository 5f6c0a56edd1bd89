"""Experiments: long runs with collectors and checkpoints (src/experiments.jl).

The reference calls ``step!``, ``collect`` and ``check_checkpoint`` after every
step (src/experiments.jl:94-144). Here the host schedules those events
instead: from the time accumulation of the reference (``time += dt`` per step,
src/integration.jl:500-503) it computes how many steps remain until the next
collector save, checkpoint or the final time, runs them on the GPU in one
``mavi_step`` call (graph launches back to back), and downloads the state only
at event times. The event steps are exactly the reference's, because the
schedule replays its floating-point time sums and comparisons.

Collectors: ``DelayedCfg`` (src/experiments.jl:411-447) keeps the last two
saved states, one at least ``delay_time`` old; ``ManyColsCfg`` combines
collectors (src/experiments.jl:363-403). Checkpoints (src/experiments.jl:
459-520) alternate between two slots so that one is always valid; files are
NumPy archives (state arrays, time, collector state), not Julia serialisation.

``stop_func(system)`` is evaluated at event times only (the reference checks
it every step), with the state downloaded; ``check_every`` adds evaluation
points every that many steps.
"""
from __future__ import annotations

import json
import os
import pathlib
from dataclasses import dataclass, field
from typing import Callable

import numpy as np

COL_DIRNAME = "data"
FINAL_STATE_NAME = "final_state"
CHECKPOINT_DIRNAME = "checkpoint"
CHECKPOINT_INFO_NAME = "checkpoint_info.json"


@dataclass
class CheckpointCfg:
    """CheckpointCfg(delta_time, save_data) (src/experiments.jl:37-40)."""
    delta_time: float
    save_data: bool = False


@dataclass
class ExperimentCfg:
    """ExperimentCfg(tf, root, save_final_state, checkpoint_cfg) (src/experiments.jl:49-54)."""
    tf: float
    root: str
    save_final_state: bool = True
    checkpoint_cfg: CheckpointCfg | None = None


# ---------------------------------------------------------------------------
# snapshots of a system's state
# ---------------------------------------------------------------------------
def _snapshot(system):
    st = system.state
    snap = {"num_steps": int(system.time_info.num_steps), "time": float(system.time_info.time),
            "pos": np.array(st.pos, copy=True)}
    for name in ("vel", "pol", "pol_angle", "rings_pos"):
        v = getattr(st, name, None)
        if isinstance(v, np.ndarray):
            snap[name] = v.copy()
    if getattr(system, "variable_rings", False):
        # which rings are active (the rings serializer keeps the mask and
        # rebuilds the ids on load, src/rings/serder.jl:85)
        snap["active_mask"] = system.rings_ids()[0].astype(np.int8)
    return snap


def _save_snapshot(snap, path):
    path = pathlib.Path(path)
    path.mkdir(parents=True, exist_ok=True)
    np.savez(path / "state.npz", **{k: v for k, v in snap.items() if isinstance(v, np.ndarray)})
    (path / "time_info.json").write_text(json.dumps({"time": snap["time"], "num_steps": snap["num_steps"]}))


def _load_snapshot(path):
    path = pathlib.Path(path)
    with np.load(path / "state.npz") as z:
        snap = {k: z[k] for k in z.files}
    snap.update(json.loads((path / "time_info.json").read_text()))
    return snap


def _restore(system, snap):
    st = system.state
    st.pos[...] = snap["pos"]
    for name in ("vel", "pol", "pol_angle", "rings_pos"):
        if name in snap and isinstance(getattr(st, name, None), np.ndarray):
            getattr(st, name)[...] = snap[name]
    if "active_mask" in snap:
        from .rings import ActiveState
        st.active_state = ActiveState(np.asarray(snap["active_mask"]).astype(bool))
    system.time_info.time = snap["time"]
    system.time_info.num_steps = snap["num_steps"]


# ---------------------------------------------------------------------------
# collectors
# ---------------------------------------------------------------------------
@dataclass
class DelayedCfg:
    """DelayedCfg(delay_time) (src/experiments.jl:411-413)."""
    delay_time: float

    def collector(self, exp_cfg, system, state=None):
        return DelayedCol(self, system, state)


class DelayedCol:
    """Keeps the last two saved states; a new one is saved when the time since
    the last save exceeds delay_time (src/experiments.jl:415-447)."""

    def __init__(self, cfg: DelayedCfg, system, state=None):
        self.cfg = cfg
        if state is None:
            state = {"last_save_time": float(system.time_info.time), "states": [_snapshot(system)]}
        self.state = state

    def due(self, t: float) -> bool:
        return t - self.state["last_save_time"] > self.cfg.delay_time

    def next_due(self, t: float, dt: float, cap: int) -> int:
        """Steps from time t until this collector saves (the reference's
        per-step test, replayed with its float arithmetic), at most cap."""
        k = 0
        while k < cap:
            k += 1
            t = t + dt
            if t - self.state["last_save_time"] > self.cfg.delay_time:
                return k
        return cap

    def collect(self, system):
        t = float(system.time_info.time)
        if self.due(t):
            self.state["last_save_time"] = t
            self.state["states"] = (self.state["states"] + [_snapshot(system)])[-2:]

    def save_data(self, path):
        states = self.state["states"]
        oldest = min(states, key=lambda s: s["time"])
        _save_snapshot(oldest, pathlib.Path(path))


@dataclass
class ManyColsCfg:
    """ManyColsCfg(cols=dict of collector configs) (src/experiments.jl:363-403)."""
    cols: dict = field(default_factory=dict)

    def collector(self, exp_cfg, system, state=None):
        return ManyCols(self, exp_cfg, system, state)


class ManyCols:
    def __init__(self, cfg: ManyColsCfg, exp_cfg, system, state=None):
        self.cfg = cfg
        self.cols = {k: c.collector(exp_cfg, system, None if state is None else state[k])
                     for k, c in cfg.cols.items()}

    @property
    def state(self):
        return {k: c.state for k, c in self.cols.items()}

    def next_due(self, t, dt, cap):
        return min(c.next_due(t, dt, cap) for c in self.cols.values())

    def collect(self, system):
        for c in self.cols.values():
            c.collect(system)

    def save_data(self, path):
        for k, c in self.cols.items():
            c.save_data(pathlib.Path(path) / k)


# ---------------------------------------------------------------------------
# experiment
# ---------------------------------------------------------------------------
class Checkpoint:
    """Two alternating checkpoint slots (src/experiments.jl:42-47)."""

    def __init__(self, last_time: float, last_used: str = "2", is_valid=None):
        self.last_used = last_used
        self.last_time = last_time
        self.is_valid = is_valid or {"1": False, "2": False}

    def next_due(self, t: float, dt: float, delta: float, cap: int) -> int:
        k = 0
        while k < cap:
            k += 1
            t = t + dt
            if not (t - self.last_time < delta):
                return k
        return cap


class Experiment:
    """Experiment(cfg, col_cfg, system, custom_step) (src/experiments.jl:56-81)."""

    def __init__(self, cfg: ExperimentCfg, col_cfg, system, custom_step=None, collector=None, checkpoint=None):
        from .system import get_step_function
        self.cfg = cfg
        self.col_cfg = col_cfg
        self.system = system
        self.custom_step = custom_step or get_step_function(system)
        self.col = collector or col_cfg.collector(cfg, system)
        if checkpoint is None and cfg.checkpoint_cfg is not None:
            checkpoint = Checkpoint(float(system.time_info.time))
        self.checkpoint = checkpoint


MAX_STRETCH = 100_000   # steps per GPU call at most (bounds the host-side replay)


def _steps_until(t: float, dt: float, tf: float, cap: int) -> int:
    """Steps the reference's `while time < tf` loop still takes from time t
    (at most cap)."""
    k = 0
    while t < tf and k < cap:
        t = t + dt
        k += 1
    return k


def schedule(t: float, dt: float, tf: float, col, checkpoint=None, delta=None, check_every=None,
             cap: int = MAX_STRETCH) -> int:
    """Steps to run before the next event (collector save, checkpoint, final
    time or a stop_func evaluation point); 0 when the final time is reached."""
    k = _steps_until(t, dt, tf, cap)
    if k == 0:
        return 0
    k = min(k, col.next_due(t, dt, k))
    if checkpoint is not None:
        k = min(k, checkpoint.next_due(t, dt, delta, k))
    if check_every:
        k = min(k, int(check_every))
    return max(k, 1)


def _save_checkpoint(experiment):
    cp = experiment.checkpoint
    cfg = experiment.cfg
    t = float(experiment.system.time_info.time)
    cp.last_time = t
    name = "2" if cp.last_used == "1" else "1"
    cp_dir = pathlib.Path(cfg.root) / CHECKPOINT_DIRNAME
    cp.is_valid[name] = False
    _save_snapshot(_snapshot(experiment.system), cp_dir / name / "sys_state")
    (cp_dir / name / "col_state.json").write_text(json.dumps(_col_state_json(experiment.col.state)))
    if cfg.checkpoint_cfg.save_data:
        experiment.col.save_data(pathlib.Path(cfg.root) / COL_DIRNAME)
    cp.is_valid[name] = True
    cp.last_used = name
    (cp_dir / CHECKPOINT_INFO_NAME).write_text(json.dumps(
        {"last_used": cp.last_used, "last_time": cp.last_time, "is_valid": cp.is_valid}))


def _col_state_json(state):
    """Collector state for the checkpoint file (snapshots as nested lists)."""
    def conv(v):
        if isinstance(v, np.ndarray):
            return {"__array__": v.tolist(), "shape": list(v.shape)}
        if isinstance(v, dict):
            return {k: conv(x) for k, x in v.items()}
        if isinstance(v, list):
            return [conv(x) for x in v]
        return v
    return conv(state)


def _col_state_from_json(state):
    def conv(v):
        if isinstance(v, dict) and "__array__" in v:
            return np.array(v["__array__"], dtype=np.float64).reshape(v["shape"])
        if isinstance(v, dict):
            return {k: conv(x) for k, x in v.items()}
        if isinstance(v, list):
            return [conv(x) for x in v]
        return v
    return conv(state)


def run_experiment(experiment: Experiment, stop_func: Callable | None = None, check_every: int | None = None):
    """run_experiment (src/experiments.jl:94-144) with GPU stretches between events."""
    system = experiment.system
    cfg = experiment.cfg
    col = experiment.col
    root = pathlib.Path(cfg.root)
    (root / COL_DIRNAME).mkdir(parents=True, exist_ok=True)
    # checkpoints only when the configuration asks for them
    cp = experiment.checkpoint if cfg.checkpoint_cfg is not None else None
    if cp is not None:
        for n in ("1", "2"):
            (root / CHECKPOINT_DIRNAME / n).mkdir(parents=True, exist_ok=True)
    dt = float(system.int_cfg.dt)
    delta = cfg.checkpoint_cfg.delta_time if cp is not None else None
    while True:
        k = schedule(float(system.time_info.time), dt, cfg.tf, col, cp, delta, check_every)
        if k == 0:
            break
        system.run(k, experiment.custom_step)          # one mavi_step(k); state downloaded once
        col.collect(system)
        if cp is not None:
            t = float(system.time_info.time)
            if not (t - cp.last_time < delta):
                _save_checkpoint(experiment)
        if stop_func is not None and stop_func(system):
            break
    col.save_data(root / COL_DIRNAME)
    if cfg.save_final_state:
        _save_snapshot(_snapshot(system), root / FINAL_STATE_NAME)
    (root / ".done").write_text("Experiment concluded\n")


def load_experiment(root, system, col_cfg, exp_cfg: ExperimentCfg | None = None, custom_step=None) -> Experiment:
    """load_experiment (src/experiments.jl:486-520): the latest valid
    checkpoint restored into `system` (built with the same configuration)."""
    root = pathlib.Path(root)
    info_path = root / CHECKPOINT_DIRNAME / CHECKPOINT_INFO_NAME
    if not info_path.is_file():
        raise FileNotFoundError(f"Checkpoint info file does not exist at {info_path}")
    info = json.loads(info_path.read_text())
    cp = Checkpoint(info["last_time"], info["last_used"], info["is_valid"])
    name = cp.last_used
    if not cp.is_valid[name]:
        name = "2" if name == "1" else "1"
        if not cp.is_valid[name]:
            raise RuntimeError("Every checkpoint is corrupted!")
    path = root / CHECKPOINT_DIRNAME / name
    _restore(system, _load_snapshot(path / "sys_state"))
    system.upload()
    col_state = _col_state_from_json(json.loads((path / "col_state.json").read_text()))
    exp_cfg = exp_cfg or ExperimentCfg(tf=float("inf"), root=str(root))
    col = col_cfg.collector(exp_cfg, system, col_state)
    return Experiment(exp_cfg, col_cfg, system, custom_step, collector=col, checkpoint=cp)
