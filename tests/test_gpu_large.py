"""Parity at the benchmark sizes, through size-independent properties.

At 262,144 and 4,194,304 particles the oracle still finishes in seconds for a
force evaluation and a chunk rebuild, so these tests compare chunk sets
(bit-exact) and forces (FP64 1e-12, mixed 1e-5 of the RMS force) on the full
workloads after the GPU has advanced them, plus conservation laws that hold at
any size: the pair sum of a periodic system is zero (Newton's third law)."""
import os

import numpy as np
import pytest

from helpers import rel_force_err

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 1


def chunks_equal(a, b):
    ca, ma = a
    cb, mb = b
    return np.array_equal(ca, cb) and np.array_equal(ma, mb)


@pytest.fixture(scope="module")
def wl(mg):
    from mavi_gb300 import workloads
    return workloads


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lj_4194304_chunks_forces_momentum(mg, orc, wl, precision):
    s, step = wl.lj_4194304(precision=precision)
    mg.run_system(s, num_steps=20, step_func=step)
    assert s.time_info.num_steps == 20
    ref = orc.from_system(s, nthreads=NT, step_kind=step.kind)
    assert chunks_equal(s.chunks(), ref.chunks())
    f = s.calc_forces()
    fr = ref.forces(orc.THREADED)
    err = rel_force_err(f, fr)
    assert err < (1e-12 if precision == "fp64" else 1e-5), err
    # periodic LJ: pair forces cancel in the sum
    net = np.linalg.norm(f.sum(axis=0)) / np.abs(f).sum()
    assert net < (1e-12 if precision == "fp64" else 1e-6), net
    ref.close()
    s.close()


def test_harm_262144_fp64_trajectory_and_mixed_forces(mg, orc, wl):
    s, step = wl.harm_262144(precision="fp64")
    ref = orc.from_system(s, nthreads=NT, step_kind=step.kind)
    mg.run_system(s, num_steps=50, step_func=step)
    ref.step(50, orc.THREADED)
    p = ref.state()[0]
    d = s.state.pos - p
    L = s.space_cfg.geometry_cfg.length
    d -= L * np.round(d / L)        # a particle may sit on the other side of a periodic seam
    assert np.max(np.abs(d)) < 1e-9
    ref.set_state(s.state.pos)
    ref.update_chunks()
    assert chunks_equal(s.chunks(), ref.chunks())
    # mixed form on the same relaxed state
    m = wl.harm_system(s.state.pos, L, "mixed")
    err = rel_force_err(m.calc_forces(), ref.forces(orc.THREADED))
    assert err < 1e-5, err
    mg.run_system(m, num_steps=100, step_func=step)
    ref.set_state(m.state.pos)
    ref.update_chunks()
    assert chunks_equal(m.chunks(), ref.chunks())
    for x in (s, m):
        x.close()
    ref.close()


def test_lj_batch_replicas_chunks_and_forces(mg, orc, wl):
    systems, step = wl.lj_batch(num_replicas=24, precision="mixed", n_max=20000,
                                quadrants=("rigid_rect", "periodic_rect", "rigid_circle"))
    b = mg.SystemBatch(systems, step)
    b.run(100)
    forces = b.calc_forces()
    for k, s in enumerate(systems):
        ref = orc.from_system(s, nthreads=NT, step_kind=step.kind)
        assert chunks_equal(b.handle.chunks(k), ref.chunks()), k
        err = rel_force_err(forces[k], ref.forces(orc.THREADED))
        assert err < 1e-5, (k, err)
        ref.close()
    b.close()


def test_rings_batch_device_noise_runs_and_chunks(mg, orc, wl):
    systems, _ = wl.rings_batch(num_replicas=6, rings_min=50, rings_max=300, precision="mixed")
    b = mg.SystemBatch(systems)
    b.run(200)
    for k, s in enumerate(systems):
        assert np.all(np.isfinite(s.state.rings_pos))
        ref = orc.from_system(s, nthreads=NT)
        assert chunks_equal(b.handle.chunks(k), ref.chunks()), k
        ref.forces(orc.THREADED)          # the ring areas are formed with the forces
        areas = ref.areas(s.state.num_rings)
        assert np.all(areas > 0)
        ref.close()
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lj_batch_512_every_replica(mg, orc, wl, precision):
    """The 512-replica batch of the benchmark at its full shape (7,871,648
    particles; every wall x geometry quadrant, periodic walls on circles
    included) after 100 velocity-Verlet steps of the whole batch: per replica
    the chunk sets are bit-exact and the forces agree with the oracle (FP64
    1e-12, mixed 1e-5 of the replica's RMS force). Particles start at least
    0.7 inside the circles, so within 100 steps of dt = 1e-3 none reaches the
    edge of a periodic circle's chunk grid (the reference's BoundsError)."""
    systems, step = wl.lj_batch(precision=precision)
    assert len(systems) == 512
    kinds = {(type(s.space_cfg.wall_type).__name__, type(s.space_cfg.geometry_cfg).__name__) for s in systems}
    assert len(kinds) == 4
    b = mg.SystemBatch(systems, step)
    b.run(100)
    assert all(s.time_info.num_steps == 100 for s in systems)
    forces = b.calc_forces()
    tol = 1e-12 if precision == "fp64" else 1e-5
    worst = 0.0
    for k, s in enumerate(systems):
        ref = orc.from_system(s, nthreads=NT, step_kind=step.kind)
        assert chunks_equal(b.handle.chunks(k), ref.chunks()), k
        err = rel_force_err(forces[k], ref.forces(orc.THREADED))
        worst = max(worst, err)
        assert err < tol, (k, err)
        ref.close()
    print(f"lj_batch_512 {precision}: worst replica force error {worst:.3e}")
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rings_64_every_replica(mg, orc, wl, precision):
    """The 64-replica ring-mixture batch of the benchmark at its full shape
    (1,868,100 particles) after 100 steps with device noise: per replica the
    chunk sets are bit-exact, the forces (pair, springs, area, bending,
    container) agree with the oracle and so do the ring areas of that force
    evaluation."""
    systems, _ = wl.rings_batch(precision=precision)
    assert len(systems) == 64
    b = mg.SystemBatch(systems)
    b.run(100)
    forces = b.calc_forces()
    ftol = 1e-12 if precision == "fp64" else 1e-5
    atol = 1e-10 if precision == "fp64" else 1e-5
    for k, s in enumerate(systems):
        assert np.all(np.isfinite(s.state.rings_pos))
        ref = orc.from_system(s, nthreads=NT)
        assert chunks_equal(b.handle.chunks(k), ref.chunks()), k
        fr = ref.forces(orc.THREADED)
        err = rel_force_err(forces[k], fr)
        assert err < ftol, (k, err)
        a, ra = s.areas(), ref.areas(s.state.num_rings)
        assert np.max(np.abs(a - ra) / np.abs(ra)) < atol, k
        ref.close()
    b.close()


def test_lj_4194304_energy_and_pair_distribution_mixed_follow_fp64(mg, wl):
    """The 4,194,304-particle periodic LJ state (velocity Verlet, dt = 5e-4)
    over 2,000 steps from the same start in both forms. Trajectories diverge
    chaotically, so the forms are compared on the conserved quantity and on
    the structure: the total-energy series (device-side, every 200 steps) and
    its drift agree to 1e-6 of the total energy, and the final g(r) (bins of
    0.02 up to 2.5) agree within five standard deviations of the counting
    noise of two independent samples, sqrt(n_fp64 + n_mixed) per bin."""
    from mavi_gb300 import workloads
    series, hist = {}, {}
    r_max, nb = 2.5, 125
    for precision in ("fp64", "mixed"):
        s, step = wl.lj_4194304(precision=precision)
        e0 = sum(s.energies())
        ke, pe = s.energy_series(10, 200, step)
        series[precision] = np.concatenate([[e0], ke + pe])
        hist[precision] = s.pair_distribution(r_max, nb).astype(np.float64)
        n, area = s.num_slots, s.space_cfg.geometry_cfg.length ** 2
        s.close()
    e64, emx = series["fp64"], series["mixed"]
    scale = np.abs(e64).max()
    d64 = (e64[-1] - e64[0]) / scale
    dmx = (emx[-1] - emx[0]) / scale
    _, g64 = mg.pair_correlation(hist["fp64"], r_max, n, area)
    _, gmx = mg.pair_correlation(hist["mixed"], r_max, n, area)
    noise = np.sqrt(hist["fp64"] + hist["mixed"]) * (g64 / np.maximum(hist["fp64"], 1))
    linf = float(np.max(np.abs(gmx - g64)))
    print(f"lj_4194304 over 2000 steps: energy drift fp64 {d64:.3e}, mixed {dmx:.3e}, "
          f"max series difference {np.max(np.abs(emx - e64)) / scale:.3e}; g(r) L-inf difference {linf:.3e}, "
          f"largest 5-sigma counting bound {float(np.max(5 * noise)):.3e}")
    assert np.max(np.abs(emx - e64)) / scale < 1e-6
    assert abs(dmx - d64) < 1e-6
    assert np.all(np.abs(gmx - g64) <= 5 * noise + 1e-12)


def test_lj_1024_fp64_trajectory_all_2000_steps(mg, orc, wl):
    """The CPU-runnable configuration over its full length: 1,024 LJ particles
    in a rigid box, velocity Verlet dt = 1e-3, 2,000 steps. The FP64 form
    follows the oracle's trajectory (same arithmetic up to the summation order
    of the pair terms) to 1e-8, and its chunk lists at the end are the
    oracle's."""
    s, step = wl.lj_1024(precision="fp64")
    ref = orc.from_system(s, step_kind=step.kind)
    mg.run_system(s, num_steps=2000, step_func=step)
    ref.step(2000)
    p, v, _ = ref.state()
    assert np.max(np.abs(s.state.pos - p)) < 1e-8
    assert np.max(np.abs(s.state.vel - v)) < 1e-8
    ref.update_chunks()
    assert chunks_equal(s.chunks(), ref.chunks())
    ref.close()
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lj_16777216_largest_single_system(mg, orc, wl, precision):
    """The largest single system tested: the LJ grid at 4096 x 4096 (16,777,216
    particles, 4.9 M chunks, periodic), four times the largest configuration.
    After 10 steps the chunk lists are the oracle's, bit for bit, and the
    forces agree (FP64 1e-12, mixed 1e-5 of the RMS force)."""
    s, step = wl.lj_4194304(precision=precision, side=4096)
    assert s.num_slots == 16777216
    mg.run_system(s, num_steps=10, step_func=step)
    ref = orc.from_system(s, nthreads=NT, step_kind=step.kind)
    assert chunks_equal(s.chunks(), ref.chunks())
    err = rel_force_err(s.calc_forces(), ref.forces(orc.THREADED))
    assert err < (1e-12 if precision == "fp64" else 1e-5), err
    ref.close()
    s.close()
