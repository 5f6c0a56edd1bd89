"""The JSON cache of the pair-pass autotuner's choices (mavi_gb300/tuning.py)."""
import json

import numpy as np
import pytest

from helpers import lj_grid, soft_disks


def test_shape_key_and_cache_round_trip(mg, tmp_path):
    from mavi_gb300 import tuning
    a = soft_disks(mg, 1024, precision="mixed")
    b = soft_disks(mg, 1100, precision="mixed")     # the same half-octave buckets
    c = lj_grid(mg, 32, 32, precision="mixed")
    ka = tuning.shape_key([a], mg.overdamped_step.kind, "mixed")
    assert ka == tuning.shape_key([b], mg.overdamped_step.kind, "mixed")
    assert ka != tuning.shape_key([c], mg.newton_step.kind, "mixed")
    assert ka != tuning.shape_key([a], mg.overdamped_step.kind, "fp64")
    cache = tuning.TuneCache(tmp_path / "tune.json")
    assert cache.get(ka) is None
    cache.put(ka, 7)
    cache.put("other", 2)
    assert cache.get(ka) == 7 and cache.get("other") == 2
    d = json.loads((tmp_path / "tune.json").read_text())
    assert d["version"] == 1 and d["entries"][ka] == {"gather_mode": 7, "gather": "split"}
    (tmp_path / "tune.json").write_text("not json")      # a damaged file reads as empty
    assert cache.get(ka) is None


def test_tuned_options_take_the_cached_mode(mg, tmp_path):
    from mavi_gb300 import tuning
    s = soft_disks(mg, 1024, precision="mixed")
    dev = mg.CUDADevice("mixed", tune_cache=str(tmp_path / "t.json"))
    kind = mg.overdamped_step.kind
    opt, cache, key = tuning.tuned_options([s], kind, dev)
    assert opt.gather_mode == -1 and cache is not None and key == tuning.shape_key([s], kind, "mixed")
    cache.put(key, 2)
    opt, cache, key = tuning.tuned_options([s], kind, dev)
    assert opt.gather_mode == 2 and cache is None and key is None
    pinned = mg.CUDADevice("mixed", gather="global", tune_cache=str(tmp_path / "t.json"))
    opt, cache, key = tuning.tuned_options([s], kind, pinned)
    assert opt.gather_mode == 1 and cache is None


@pytest.mark.gpu
def test_cache_records_then_reuses_the_choice(mg, tmp_path):
    """The first handle of a shape is autotuned and records its mode; the
    second is created with that mode (no timing) and gives the same bits."""
    path = tmp_path / "tune.json"
    runs = []
    for _ in range(2):
        s = soft_disks(mg, 8192, precision="mixed")
        s.int_cfg.device.tune_cache = str(path)
        mg.run_system(s, num_steps=20, step_func=mg.overdamped_step)   # the handle (one shape key)
        f = s.calc_forces()
        runs.append((f, s.state.pos.copy(), s.stats().gather_mode))
        s.close()
    entries = json.loads(path.read_text())["entries"]
    assert len(entries) == 1 and list(entries.values())[0]["gather_mode"] == runs[0][2]
    assert runs[0][2] == runs[1][2]
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])
