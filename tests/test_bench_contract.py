"""bench.py's reference arm prints one JSON line with the fields the benchmark
contract asks for (CPU only: the reference arm runs the oracle port)."""
import json
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "lj_1024",
                        "--steps", "3", "--warmup", "1"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["workload"] == "lj_1024"


def test_cpu_baseline_at_one_core_and_all_cores(mg, orc):
    """The CPU baseline leg times whole replicas of the workload through the
    oracle, sequential at one thread and column-split threaded above."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    from helpers import lj_grid

    class FakeRunner:           # the attributes cpu_baseline reads, no device handle
        def __init__(self, systems):
            self.systems = systems
            self.kind = mg.abi.MAVI_STEP_NEWTON
            self.num_slots = sum(s.num_slots for s in systems)

    r = FakeRunner([lj_grid(mg, 16, 16, chunks=(6, 6))])
    for nthreads in (1, 2):
        out = bench.cpu_baseline(mg, orc, r, 0.2, nthreads)
        assert out["value"] > 0 and out["cores"] == nthreads and out["kind"] == "port"
        assert ("Threaded" in out["sample"]) == (nthreads > 1)


def test_gather_option_pins_the_mixed_form_only(mg):
    """--gather pins the mixed form's pair gather (profiling runs); the FP64
    form keeps the autotuner."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod2", ROOT / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    bench.MIXED_GATHER = "split"
    mixed, _ = bench.workload_share("lj_1024", "mixed")
    fp64, _ = bench.workload_share("lj_1024", "fp64")
    assert mixed.int_cfg.device.gather == "split" and fp64.int_cfg.device.gather == "auto"
    assert mixed.int_cfg.device.options().gather_mode == 7
