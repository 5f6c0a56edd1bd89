"""The tiled Newton's-third-law pass of the mixed Lennard-Jones / WCA forms.

Every pair with an owned particle is evaluated once per tile of chunks and
added to both particles (halo partners: to the owned one only). Force sums are
fixed point in shared memory, so the two tiled modes (a CTA per tile, and
persistent CTAs on a device work queue) give the same bits and every run
gives the same bits; against the per-particle gathers and the oracle the
forces agree within the mixed tolerance (1e-5 of the RMS force)."""
import os

import numpy as np
import pytest

from helpers import lj_grid, rel_force_err, self_propelled, soft_disks

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1
TOL = 1e-5


def _batch(mg, gather, **kw):
    from mavi_gb300 import workloads
    systems, step = workloads.lj_batch(precision="mixed", **kw)
    for s in systems:
        s.int_cfg.device.gather = gather
    return systems, step


def _run(mg, gather, steps=60, **kw):
    systems, step = _batch(mg, gather, **kw)
    b = mg.SystemBatch(systems, step)
    f = np.concatenate(b.calc_forces())
    b.run(steps)
    mode = b.handle.stats().gather_mode
    pos = np.concatenate([s.state.pos for s in systems])
    vel = np.concatenate([s.state.vel for s in systems])
    b.close()
    return f, pos, vel, mode


def test_tile_modes_agree_bitwise_and_are_deterministic(mg):
    """Both tiled modes, twice each, on a batch with all four wall x geometry
    quadrants (edge tiles, wrapped halos, periodic circles with raw far
    pairs): forces and 60-step trajectories identical bit for bit."""
    kw = dict(num_replicas=8, n_min=600, n_max=6000)
    runs = [_run(mg, g, **kw) for g in ("tiles", "tiles_queue", "tiles", "tiles_queue")]
    assert [r[3] for r in runs] == [3, 4, 3, 4]
    for r in runs[1:]:
        for a, c in zip(runs[0][:3], r[:3]):
            assert np.array_equal(a, c)


def test_tiles_match_the_gather(mg):
    kw = dict(num_replicas=8, n_min=600, n_max=6000)
    ft, _, _, _ = _run(mg, "tiles", steps=0, **kw)
    fg, _, _, _ = _run(mg, "global", steps=0, **kw)
    assert rel_force_err(ft, fg) < 1e-6


@pytest.mark.parametrize("gather", ["tiles", "tiles_queue"])
def test_tiles_forces_against_oracle(mg, orc, gather):
    systems, step = _batch(mg, gather, num_replicas=12, n_min=1000, n_max=20000)
    b = mg.SystemBatch(systems, step)
    b.run(50)
    forces = b.calc_forces()
    for k, s in enumerate(systems):
        ref = orc.from_system(s, nthreads=NT, step_kind=step.kind)
        err = rel_force_err(forces[k], ref.forces(orc.THREADED))
        assert err < TOL, (k, err)
        ref.close()
    b.close()


@pytest.mark.parametrize("chunks", [(3, 3), (4, 4), (5, 7)])
def test_tiles_on_small_periodic_grids(mg, orc, chunks):
    """Grids no wider than a tile: halo columns and rows are wrapped copies of
    the tile's own chunks; those pairs are evaluated from both sides."""
    s = lj_grid(mg, 12, 12, wall="periodic", chunks=chunks, precision="mixed")
    s.int_cfg.device.gather = "tiles_queue"
    ref = orc.from_system(s)
    assert rel_force_err(s.calc_forces(), ref.forces()) < TOL
    mg.run_system(s, num_steps=100)
    ref.step(100)
    assert np.max(np.abs(s.state.pos - ref.state()[0])) < 1e-5
    ref.close()
    s.close()


def test_tiles_fall_back_for_dense_windows(mg, orc):
    """A crystal patch (spacing 1) in a dilute gas: the mean density makes
    large tiles, whose windows over the patch exceed the shared-memory arrays
    and run the per-particle gather instead; forces still match the oracle."""
    rng = np.random.default_rng(5)
    L = 120.0
    g = np.arange(40) * 1.0 + 10.0                    # crystal patch, spacing 1, in [10, 49]^2
    dense = np.stack(np.meshgrid(g, g), axis=-1).reshape(-1, 2)
    h = (np.arange(40) + 0.5) * 3.0                   # gas: spacing 3 outside the patch, jittered
    gas = np.stack(np.meshgrid(h, h), axis=-1).reshape(-1, 2)
    gas = gas[~((gas[:, 0] > 7) & (gas[:, 0] < 53) & (gas[:, 1] > 7) & (gas[:, 1] < 53))]
    gas = gas + rng.uniform(-0.3, 0.3, gas.shape)
    pos = np.concatenate([dense, gas])
    out = []
    for gather in ("global", "tiles", "tiles_queue"):
        s = mg.System(mg.SecondLawState(pos.copy(), np.zeros_like(pos)),
                      mg.SpaceCfg(mg.PeriodicWalls(), mg.RectangleCfg(L, L)), mg.LenJonesCfg(1.0, 1.0),
                      mg.IntCfg(dt=1e-4, chunks_cfg=mg.ChunksCfg(48, 48),
                                device=mg.CUDADevice(precision="mixed", gather=gather)))
        f = s.calc_forces()
        ref = orc.from_system(s)
        assert rel_force_err(f, ref.forces()) < TOL, gather
        ref.close()
        mg.run_system(s, num_steps=20)
        out.append(s.state.pos.copy())
        s.close()
    assert np.array_equal(out[1], out[2])
    assert np.max(np.abs(out[0] - out[1])) < 1e-9


def test_tiles_run_and_tumble_against_oracle(mg, orc):
    """WCA (run-and-tumble) with injected noise: tiled trajectory against the oracle."""
    s = self_propelled(mg, "rtp", n=900, precision="mixed", noise="injected")
    s.int_cfg.device.gather = "tiles"
    ref = orc.from_system(s)
    assert rel_force_err(s.calc_forces(), ref.forces()) < TOL
    n = s._ensure().noise_count()
    steps = 30
    noise = np.random.default_rng(2).random(n * steps)
    s.run(steps, noise=noise)
    ref.step(steps, noise=noise)
    assert np.max(np.abs(s.state.pos - ref.state()[0])) < 1e-4
    ref.close()
    s.close()


def test_tiles_reject_other_laws(mg):
    s = soft_disks(mg, 2000, precision="mixed")
    s.int_cfg.device.gather = "tiles"
    with pytest.raises(mg.MaviError) as e:
        s.calc_forces()
    assert e.value.status == mg.abi.MAVI_ERR_UNSUPPORTED
