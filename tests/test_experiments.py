"""The experiment loop (src/experiments.jl): events happen at exactly the
reference's steps although the steps between events run in one call, and a
run resumed from a checkpoint ends in the same state."""
import json
import types

import numpy as np
import pytest

from helpers import lj_grid


class FakeSystem:
    """Host-only stand-in: run(k) advances the time like System.run and
    changes the state deterministically (no GPU)."""

    def __init__(self, dt):
        self.int_cfg = types.SimpleNamespace(dt=dt)
        self.time_info = types.SimpleNamespace(time=0.0, num_steps=0)
        self.state = types.SimpleNamespace(pos=np.zeros((3, 2)), vel=np.zeros((3, 2)))
        self.calls = []

    def run(self, k, step_func=None):
        self.calls.append(k)
        for _ in range(k):
            self.time_info.time += self.int_cfg.dt
            self.time_info.num_steps += 1
            self.state.pos += 1.0

    def upload(self):
        pass


def reference_loop(dt, tf, delay, delta):
    """The reference's per-step loop: the times at which DelayedCol saves and
    check_checkpoint writes (src/experiments.jl:120-127, 430-440, 459-470)."""
    t, last_save, last_cp = 0.0, 0.0, 0.0
    saves, cps = [], []
    while t < tf:
        t += dt
        if t - last_save > delay:
            last_save = t
            saves.append(t)
        if not (t - last_cp < delta):
            last_cp = t
            cps.append(t)
    return saves, cps, t


@pytest.mark.parametrize("dt,tf,delay,delta", [(1e-3, 0.5, 0.0317, 0.1), (0.01, 3.0, 0.25, 0.7), (0.1, 1.0, 0.0, 0.3)])
def test_event_steps_match_the_reference_loop(mg, tmp_path, dt, tf, delay, delta):
    ex = mg.experiments
    sys_ = FakeSystem(dt)
    saves_seen, cps_seen = [], []
    exp = ex.Experiment(ex.ExperimentCfg(tf=tf, root=str(tmp_path), checkpoint_cfg=ex.CheckpointCfg(delta)),
                        ex.DelayedCfg(delay), sys_, custom_step=types.SimpleNamespace(kind=0))
    orig_collect = exp.col.collect

    def collect(system):
        before = exp.col.state["last_save_time"]
        orig_collect(system)
        if exp.col.state["last_save_time"] != before:
            saves_seen.append(system.time_info.time)
    exp.col.collect = collect
    orig_save = ex._save_checkpoint

    def save(e):
        cps_seen.append(e.system.time_info.time)
        orig_save(e)
    ex._save_checkpoint = save
    try:
        ex.run_experiment(exp)
    finally:
        ex._save_checkpoint = orig_save
    saves, cps, t_end = reference_loop(dt, tf, delay, delta)
    assert saves_seen == saves
    assert cps_seen == cps
    assert sys_.time_info.time == t_end
    assert len(sys_.calls) <= len(saves) + len(cps) + 1    # one call per event stretch
    assert (tmp_path / ".done").exists() and (tmp_path / "final_state" / "state.npz").exists()


@pytest.mark.gpu
def test_experiment_on_gpu_and_resume_from_checkpoint(mg, tmp_path):
    ex = mg.experiments
    tf, dt = 0.35, 1e-3
    s = lj_grid(mg, 16, 16, wall="periodic", dt=dt)
    exp = ex.Experiment(ex.ExperimentCfg(tf=tf, root=str(tmp_path / "a"), checkpoint_cfg=ex.CheckpointCfg(0.1)),
                        ex.DelayedCfg(0.05), s)
    ex.run_experiment(exp)
    full = s.state.pos.copy()
    n_full = s.time_info.num_steps
    s.close()
    # the same number of steps in one run_system call gives the same state
    r = lj_grid(mg, 16, 16, wall="periodic", dt=dt)
    mg.run_system(r, num_steps=n_full)
    assert np.array_equal(r.state.pos, full)
    r.close()
    # resume from the last checkpoint and finish
    info = json.loads((tmp_path / "a" / "checkpoint" / "checkpoint_info.json").read_text())
    assert info["is_valid"][info["last_used"]]
    s2 = lj_grid(mg, 16, 16, wall="periodic", dt=dt)
    exp2 = ex.load_experiment(tmp_path / "a", s2, ex.DelayedCfg(0.05), ex.ExperimentCfg(tf=tf, root=str(tmp_path / "b")))
    assert s2.time_info.num_steps < n_full
    ex.run_experiment(exp2)
    assert s2.time_info.num_steps == n_full
    assert np.array_equal(s2.state.pos, full)
    s2.close()


def _fake_experiment(ex, root, dt=0.01, tf=1.0, delta=0.2):
    s = FakeSystem(dt)
    e = ex.Experiment(ex.ExperimentCfg(tf=tf, root=str(root), checkpoint_cfg=ex.CheckpointCfg(delta)),
                      ex.DelayedCfg(0.05), s, custom_step=types.SimpleNamespace(kind=0))
    return s, e


def test_crash_while_writing_a_checkpoint_resumes_from_the_last_complete_one(mg, tmp_path):
    """Host-side fault injection (as test/tests_experiments.jl:60-65 does with
    an `error`): the third checkpoint write fails half-way; the info file still
    names the last complete checkpoint, and a resumed run ends where an
    uninterrupted one does."""
    ex = mg.experiments
    orig = ex._save_snapshot
    calls = {"n": 0}

    def failing(snap, path):
        if "checkpoint" in str(path):
            calls["n"] += 1
            if calls["n"] == 3:
                raise RuntimeError("injected failure while writing a checkpoint")
        return orig(snap, path)
    ex._save_snapshot = failing
    try:
        s, e = _fake_experiment(ex, tmp_path / "a")
        with pytest.raises(RuntimeError, match="injected"):
            ex.run_experiment(e)
    finally:
        ex._save_snapshot = orig
    info = json.loads((tmp_path / "a" / "checkpoint" / "checkpoint_info.json").read_text())
    assert info["is_valid"] == {"1": True, "2": True}
    s2 = FakeSystem(0.01)
    e2 = ex.load_experiment(tmp_path / "a", s2, ex.DelayedCfg(0.05), custom_step=types.SimpleNamespace(kind=0))
    assert s2.time_info.time == info["last_time"]
    assert np.all(s2.state.pos == s2.time_info.num_steps)          # the state of that checkpoint
    e2.cfg = ex.ExperimentCfg(tf=1.0, root=str(tmp_path / "b"), checkpoint_cfg=ex.CheckpointCfg(0.2))
    ex.run_experiment(e2)
    ref, ref_e = _fake_experiment(ex, tmp_path / "c")
    ex.run_experiment(ref_e)
    assert s2.time_info.num_steps == ref.time_info.num_steps
    assert np.array_equal(s2.state.pos, ref.state.pos)


def test_invalid_checkpoints_are_skipped_or_refused(mg, tmp_path):
    """load_experiment (src/experiments.jl:490-520): the last used checkpoint
    if valid, else the other one; neither valid is an error."""
    ex = mg.experiments
    s, e = _fake_experiment(ex, tmp_path)
    ex.run_experiment(e)
    path = tmp_path / "checkpoint" / "checkpoint_info.json"
    info = json.loads(path.read_text())
    last, other = info["last_used"], ("2" if info["last_used"] == "1" else "1")
    times = {}
    for name in ("1", "2"):
        info2 = dict(info, last_used=name, is_valid={"1": True, "2": True})
        path.write_text(json.dumps(info2))
        s2 = FakeSystem(0.01)
        ex.load_experiment(tmp_path, s2, ex.DelayedCfg(0.05), custom_step=types.SimpleNamespace(kind=0))
        times[name] = s2.time_info.time
    assert times[last] > times[other]
    path.write_text(json.dumps(dict(info, is_valid={last: False, other: True})))
    s3 = FakeSystem(0.01)
    ex.load_experiment(tmp_path, s3, ex.DelayedCfg(0.05), custom_step=types.SimpleNamespace(kind=0))
    assert s3.time_info.time == times[other]
    path.write_text(json.dumps(dict(info, is_valid={"1": False, "2": False})))
    with pytest.raises(RuntimeError, match="corrupted"):
        ex.load_experiment(tmp_path, FakeSystem(0.01), ex.DelayedCfg(0.05))
    path.unlink()
    with pytest.raises(FileNotFoundError):
        ex.load_experiment(tmp_path, FakeSystem(0.01), ex.DelayedCfg(0.05))
