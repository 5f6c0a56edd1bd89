"""Long-run statistics on the GPU: the pair-distance histogram behind g(r)
(exact integer counts, equal to the oracle's) and the device-side energy
series (equal to stepping and measuring in turn)."""
import math
import os

import numpy as np
import pytest

from helpers import lj_grid

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pair_distribution_equals_oracle(mg, orc, precision):
    """The 512 x 512 LJ grid state (262,144 particles, periodic) after 20
    Verlet steps: every bin of the GPU histogram equals the oracle's count on
    the downloaded positions."""
    from mavi_gb300 import workloads
    s, step = workloads.lj_262144(precision=precision)
    mg.run_system(s, num_steps=20, step_func=step)
    r_max = 2.5
    counts = s.pair_distribution(r_max, 250)
    ref = orc.from_system(s, nthreads=NT, step_kind=step.kind)
    rc = ref.pair_distribution(r_max, 250)
    assert counts.sum() > 0
    assert np.array_equal(counts, rc)
    r, g = mg.pair_correlation(counts, r_max, s.num_slots, s.space_cfg.geometry_cfg.length ** 2)
    assert g[r < 0.8].max() == 0 and g.max() > 1.5          # no overlaps; a first-shell peak
    ref.close()
    s.close()


def test_pair_distribution_of_a_batch(mg, orc):
    """Every quadrant of the replica batch: per replica and summed (-1)."""
    from mavi_gb300 import workloads
    systems, step = workloads.lj_batch(num_replicas=8, n_min=800, n_max=4000, precision="mixed")
    b = mg.SystemBatch(systems, step)
    b.run(30)
    r_max = 2.5
    total = np.zeros(100, dtype=np.uint64)
    for k, s in enumerate(systems):
        ref = orc.from_system(s, nthreads=NT, step_kind=step.kind)
        rc = ref.pair_distribution(r_max, 100)
        assert np.array_equal(b.pair_distribution(r_max, 100, replica=k), rc), k
        total += rc
        ref.close()
    assert np.array_equal(b.pair_distribution(r_max, 100), total)
    b.close()


def test_pair_distribution_rejects_r_max_beyond_chunks(mg):
    s = lj_grid(mg, 12, 12, wall="periodic", chunks=(5, 5))
    with pytest.raises(mg.MaviError) as e:
        s.pair_distribution(10.0, 10)
    assert e.value.status == mg.abi.MAVI_ERR_INVALID_ARG
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_energy_series_equals_stepping_and_measuring(mg, precision):
    """The device-side series gives, bit for bit, what stepping and calling
    mavi_energies in turn gives."""
    a = lj_grid(mg, 20, 20, wall="periodic", precision=precision)
    b = lj_grid(mg, 20, 20, wall="periodic", precision=precision)
    for s in (a, b):   # one gather for both (the autotuner may time two choices differently)
        s.int_cfg.device.gather = "global"
    ke, pe = a.energy_series(5, 40)
    seq = []
    for _ in range(5):
        mg.run_system(b, num_steps=40)
        seq.append(b.energies())
    seq = np.array(seq)
    assert np.array_equal(ke, seq[:, 0]) and np.array_equal(pe, seq[:, 1])
    assert a.time_info.num_steps == 200
    assert np.array_equal(a.state.pos, b.state.pos)
    a.close()
    b.close()
