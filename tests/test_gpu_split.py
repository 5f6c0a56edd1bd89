"""The split gather of the mixed Lennard-Jones passes (pass mode 7).

Pairs at r >= 2 sigma are evaluated in plain FP32, closer ones in
double-float after them, each particle's terms in one fixed order: every run
gives the same bits, both particles of a pair get opposite forces, and the
forces agree with the oracle within the mixed tolerance (1e-5 of the RMS
force) and with the double-float column gather within 1e-6."""
import os

import numpy as np
import pytest

from helpers import lj_grid, rel_force_err, soft_disks

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1
TOL = 1e-5


def _batch(gather, **kw):
    from mavi_gb300 import workloads
    systems, step = workloads.lj_batch(precision="mixed", **kw)
    for s in systems:
        s.int_cfg.device.gather = gather
    return systems, step


def _run(mg, gather, steps=60, **kw):
    systems, step = _batch(gather, **kw)
    b = mg.SystemBatch(systems, step)
    f = np.concatenate(b.calc_forces())
    b.run(steps)
    mode = b.handle.stats().gather_mode
    pos = np.concatenate([s.state.pos for s in systems])
    vel = np.concatenate([s.state.vel for s in systems])
    b.close()
    return f, pos, vel, mode


def test_split_is_deterministic(mg):
    """Twice on a batch with all four wall x geometry quadrants (clipped and
    wrapped stencils, raw wrapped pairs of periodic circles): forces and
    60-step trajectories identical bit for bit."""
    kw = dict(num_replicas=8, n_min=600, n_max=6000)
    a, b = _run(mg, "split", **kw), _run(mg, "split", **kw)
    assert a[3] == 7 and b[3] == 7
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)


def test_split_matches_the_column_gather(mg):
    kw = dict(num_replicas=8, n_min=600, n_max=6000)
    fs, ps, _, _ = _run(mg, "split", steps=40, **kw)
    fc, pc, _, _ = _run(mg, "columns", steps=40, **kw)
    assert rel_force_err(fs, fc) < 1e-6
    assert np.max(np.abs(ps - pc)) < 1e-8


def test_split_forces_against_oracle(mg, orc):
    systems, step = _batch("split", num_replicas=12, n_min=1000, n_max=20000)
    b = mg.SystemBatch(systems, step)
    b.run(50)
    forces = b.calc_forces()
    for k, s in enumerate(systems):
        ref = orc.from_system(s, nthreads=NT, step_kind=step.kind)
        err = rel_force_err(forces[k], ref.forces(orc.THREADED))
        assert err < TOL, (k, err)
        ref.close()
    b.close()


@pytest.mark.parametrize("wall", ["periodic", "rigid"])
def test_split_trajectory_against_oracle(mg, orc, wall):
    """A 60 x 60 LJ lattice over 200 velocity-Verlet steps: positions within
    1e-6 of the oracle's FP64 trajectory; in the periodic box the pair forces
    cancel in the sum (opposite forces for the two particles of a pair)."""
    s = lj_grid(mg, 60, 60, wall=wall, precision="mixed", speed=1.0)
    s.int_cfg.device.gather = "split"
    ref = orc.from_system(s, nthreads=NT)
    f = s.calc_forces()
    assert s.stats().gather_mode == 7
    assert rel_force_err(f, ref.forces(orc.THREADED)) < TOL
    if wall == "periodic":
        assert np.linalg.norm(f.sum(axis=0)) / np.abs(f).sum() < 1e-6
    mg.run_system(s, num_steps=200)
    ref.step(200)
    assert np.max(np.abs(s.state.pos - ref.state()[0])) < 1e-6
    ref.close()
    s.close()


def test_split_on_a_dense_hot_state(mg, orc):
    """Close contacts (a compressed lattice, offset 0.05, heated) on a coarse
    8 x 8 chunk grid: ~320 candidates per particle, some particles with more
    close candidates than the pass parks (those take the per-chunk gather)."""
    s = lj_grid(mg, 48, 48, wall="periodic", precision="mixed", speed=2.0, offset=0.05, chunks=(8, 8))
    s.int_cfg.device.gather = "split"
    mg.run_system(s, num_steps=100)
    ref = orc.from_system(s, nthreads=NT)
    assert rel_force_err(s.calc_forces(), ref.forces(orc.THREADED)) < TOL
    ref.close()
    s.close()


def test_split_rejects_other_forms(mg):
    for s in (soft_disks(mg, 1024, precision="mixed"), lj_grid(mg, 8, 8, precision="fp64")):
        s.int_cfg.device.gather = "split"
        with pytest.raises(mg.MaviError) as e:
            s.calc_forces()
        assert e.value.status == mg.abi.MAVI_ERR_UNSUPPORTED


@pytest.mark.parametrize("wall", ["rigid", "periodic"])
def test_split_all_pairs_without_chunks(mg, orc, wall):
    """No chunk grid (every pair of the replica is a candidate, ~400 per
    particle, so most are evaluated in FP32): forces and a 50-step trajectory
    against the oracle's all-pairs form."""
    s = lj_grid(mg, 20, 20, wall=wall, chunks=False, precision="mixed")
    s.int_cfg.device.gather = "split"
    ref = orc.from_system(s)
    assert rel_force_err(s.calc_forces(), ref.forces(orc.ALL_PAIRS)) < TOL
    assert s.stats().gather_mode == 7
    mg.run_system(s, num_steps=50)
    ref.step(50)
    assert np.max(np.abs(s.state.pos - ref.state()[0])) < 1e-6
    ref.close()
    s.close()


def test_split_forces_on_a_melted_batch(mg, orc):
    """After 3,000 steps (the jittered lattices have melted into liquids at
    T = 0.3-1.0: more close pairs, disordered shells) the split gather's
    forces still agree with the oracle's FP64 forces on the same positions.
    (Periodic circles are left out: with no wall and no wrap, particles leave
    their grid within ~2,700 steps, the reference's BoundsError.)"""
    systems, step = _batch("split", num_replicas=9, n_min=2000, n_max=12000,
                           quadrants=("rigid_rect", "periodic_rect", "rigid_circle"))
    b = mg.SystemBatch(systems, step)
    b.run(3000)
    forces = b.calc_forces()
    assert b.handle.stats().gather_mode == 7
    for k, s in enumerate(systems):
        ref = orc.from_system(s, nthreads=NT, step_kind=step.kind)
        err = rel_force_err(forces[k], ref.forces(orc.THREADED))
        assert err < TOL, (k, err)
        ref.close()
    b.close()
