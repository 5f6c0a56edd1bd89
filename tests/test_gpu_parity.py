"""Parity of the CUDA library (through its C ABI) with the oracle on the same
seeded inputs. Chunk sets must be bit-exact; FP64 forces agree to 1e-12 of
the RMS force (summation order differs); mixed-precision forces to 1e-5."""
import numpy as np
import pytest

from helpers import lj_grid, soft_disks, lj_circle, self_propelled, rings_normal, rings_types, rel_force_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 1e-5


def chunks_equal(sys_, ref):
    c_gpu, m_gpu = sys_.chunks()
    c_ref, m_ref = ref.chunks()
    return np.array_equal(c_gpu, c_ref) and np.array_equal(m_gpu, m_ref)


@pytest.mark.parametrize("wall", ["rigid", "periodic"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lj_grid_chunks_and_forces(mg, orc, wall, precision):
    s = lj_grid(mg, 32, 32, wall=wall, chunks=(17, 17), precision=precision)
    ref = orc.from_system(s)
    assert chunks_equal(s, ref)
    err = rel_force_err(s.calc_forces(), ref.forces())
    assert err < (FP64_TOL if precision == "fp64" else MIXED_TOL), err
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lj_trajectory_rigid(mg, orc, precision):
    s = lj_grid(mg, 32, 32, wall="rigid", chunks=(17, 17), precision=precision)
    ref = orc.from_system(s)
    mg.run_system(s, num_steps=200)
    ref.step(200)
    p, v, _ = ref.state()
    tol = 1e-9 if precision == "fp64" else 1e-4
    assert np.max(np.abs(s.state.pos - p)) < tol
    assert np.max(np.abs(s.state.vel - v)) < tol * 10
    assert s.time_info.num_steps == 200 and ref.time()[0] == 200
    assert chunks_equal(s, ref) if precision == "fp64" else True
    s.close()


def test_lj_trajectory_periodic_chunks_bit_exact_after_steps(mg, orc):
    s = lj_grid(mg, 24, 24, wall="periodic", speed=1.0)
    ref = orc.from_system(s)
    for _ in range(4):
        mg.run_system(s, num_steps=50)
        ref.step(50)
        ref.set_state(s.state.pos, s.state.vel)   # same FP64 state on both sides
        ref.update_chunks()
        assert chunks_equal(s, ref)
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_overdamped_soft_disks(mg, orc, precision):
    s = soft_disks(mg, 4096, precision=precision)
    ref = orc.from_system(s, step_kind=mg.overdamped_step.kind)
    assert chunks_equal(s, ref)
    err = rel_force_err(s.calc_forces(), ref.forces())
    assert err < (FP64_TOL if precision == "fp64" else MIXED_TOL), err
    mg.run_system(s, num_steps=50, step_func=mg.overdamped_step)
    ref.step(50)
    tol = 1e-9 if precision == "fp64" else 1e-4
    assert np.max(np.abs(s.state.pos - ref.state()[0])) < tol
    s.close()


@pytest.mark.parametrize("wall", ["rigid", "slippery"])
def test_circle_walls(mg, orc, wall):
    s = lj_circle(mg, 300, wall=wall)
    ref = orc.from_system(s)
    assert chunks_equal(s, ref)
    mg.run_system(s, num_steps=100)
    ref.step(100)
    assert np.max(np.abs(s.state.pos - ref.state()[0])) < 1e-9
    s.close()


@pytest.mark.parametrize("kind", ["szabo", "rtp"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_self_propelled_injected_noise(mg, orc, kind, precision):
    s = self_propelled(mg, kind, 400, precision=precision)
    step = mg.szabo_step if kind == "szabo" else mg.rtp_step
    ref = orc.from_system(s)
    err = rel_force_err(s.calc_forces(), ref.forces())
    assert err < (FP64_TOL if precision == "fp64" else MIXED_TOL), err
    n = s.handle.noise_count()
    assert n == ref.noise_count()
    rng = np.random.default_rng(11)
    steps = 30
    noise = rng.normal(size=n * steps) if kind == "szabo" else rng.random(n * steps)
    s.run(steps, step, noise=noise)
    ref.step(steps, noise=noise)
    p, _, pol = ref.state()
    tol = 1e-9 if precision == "fp64" else 1e-4
    assert np.max(np.abs(s.state.pos - p)) < tol
    assert np.max(np.abs(s.state.pol_angle - pol)) < tol
    s.close()


@pytest.mark.parametrize("factory", ["normal", "types"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rings(mg, orc, factory, precision):
    s = rings_normal(mg, precision=precision) if factory == "normal" else rings_types(mg, precision=precision)
    ref = orc.from_system(s)
    assert chunks_equal(s, ref)
    err = rel_force_err(s.calc_forces(), ref.forces())
    assert err < (FP64_TOL if precision == "fp64" else MIXED_TOL), err
    n = s.handle.noise_count()
    steps = 100
    noise = np.random.default_rng(3).normal(size=n * steps)
    s.run(steps, noise=noise)
    ref.step(steps, noise=noise)
    p, _, pol = ref.state()
    active = np.array([k % s.state.nmax < s.state.ring_num_particles(k // s.state.nmax)
                       for k in range(s.num_slots)])
    tol = 1e-8 if precision == "fp64" else 1e-3
    assert np.max(np.abs(s.state.pos[active] - p[active])) < tol
    assert np.max(np.abs(s.state.pol - pol)) < tol
    # RingsInfo.areas: the areas of the last step's force evaluation
    a, ra = s.areas(), ref.areas(s.state.num_rings)
    assert np.max(np.abs(a - ra) / np.abs(ra)) < (1e-10 if precision == "fp64" else 1e-5)
    s.close()


@pytest.mark.parametrize("factory", ["normal", "types"])
def test_rings_column_gather_equals_global_gather_bitwise(mg, factory):
    """Mixed rings: the column-gather kernel and the per-chunk gather give the
    same forces and 50-step trajectories bit for bit."""
    out = []
    for gather in ("columns", "global"):
        s = rings_normal(mg, precision="mixed") if factory == "normal" else rings_types(mg, precision="mixed")
        s.int_cfg.device.gather = gather
        f = s.calc_forces()
        assert s.stats().gather_mode == {"columns": 2, "global": 1}[gather]
        n = s.handle.noise_count()
        s.run(50, noise=np.random.default_rng(7).normal(size=n * 50))
        out.append((f, s.state.pos.copy()))
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_rings_bending_forces(mg, orc):
    s = rings_normal(mg, k_bend=2.0)
    ref = orc.from_system(s)
    assert rel_force_err(s.calc_forces(), ref.forces()) < FP64_TOL
    s.close()


def test_all_pairs_without_chunks(mg, orc):
    s = lj_grid(mg, 10, 10, wall="rigid", chunks=False)
    ref = orc.from_system(s)
    assert rel_force_err(s.calc_forces(), ref.forces(orc.ALL_PAIRS)) < FP64_TOL
    mg.run_system(s, num_steps=50)
    ref.step(50)
    assert np.max(np.abs(s.state.pos - ref.state()[0])) < 1e-10
    s.close()


def test_energies(mg, orc):
    s = lj_grid(mg, 20, 20, wall="periodic")
    ref = orc.from_system(s)
    ke, pe = s.energies(mg.abi.MAVI_PE_STENCIL)
    rke, rpe = ref.energies(mg.abi.MAVI_PE_STENCIL)
    assert ke == pytest.approx(rke, rel=1e-13) and pe == pytest.approx(rpe, rel=1e-12)
    ke2, pe2 = s.energies(mg.abi.MAVI_PE_ALL_PAIRS)
    rke2, rpe2 = ref.energies(mg.abi.MAVI_PE_ALL_PAIRS)
    assert pe2 == pytest.approx(rpe2, rel=1e-12)
    s.close()


def test_batch_equals_single_replicas_bitwise(mg):
    singles = [lj_grid(mg, 12 + 2 * k, 12 + k, wall=("rigid" if k % 2 else "periodic"), seed=k) for k in range(4)]
    batch_sys = [lj_grid(mg, 12 + 2 * k, 12 + k, wall=("rigid" if k % 2 else "periodic"), seed=k) for k in range(4)]
    for s in singles:
        mg.run_system(s, num_steps=40)
    b = mg.SystemBatch(batch_sys)
    b.run(40)
    for s, t in zip(singles, batch_sys):
        assert np.array_equal(s.state.pos, t.state.pos)
        assert np.array_equal(s.state.vel, t.state.vel)
        s.close()
    b.close()


def test_deterministic_and_graph_equals_eager(mg):
    a = lj_grid(mg, 20, 20, wall="periodic", use_graph=True)
    b = lj_grid(mg, 20, 20, wall="periodic", use_graph=True)
    c = lj_grid(mg, 20, 20, wall="periodic", use_graph=False)
    for s in (a, b, c):
        mg.run_system(s, num_steps=100)
    assert np.array_equal(a.state.pos, b.state.pos)
    assert np.array_equal(a.state.pos, c.state.pos)
    for s in (a, b, c):
        s.close()


def test_out_of_grid_reports_error(mg):
    """A particle more than one chunk outside the grid is a BoundsError in the
    reference (src/chunks.jl:144-146); here the status is returned, no trap."""
    s = lj_grid(mg, 8, 8, wall="rigid", chunks=(4, 4))
    s.calc_forces()
    s.state.pos[5] = (-20.0, 3.0)
    s.upload()                      # queued; the next call that returns results reports it
    with pytest.raises(mg.MaviError) as e:
        s.calc_forces()
    assert e.value.status == mg.abi.MAVI_ERR_OUT_OF_GRID
    s.state.pos[5] = (1.0, 1.0)
    s.upload()                      # the handle stays usable
    s.calc_forces()
    s.close()


def test_particle_escaping_during_steps_reports_error(mg):
    s = lj_grid(mg, 8, 8, wall="periodic", chunks=(4, 4))
    s.calc_forces()
    s.state.vel[3] = (1e6, 0.0)     # crosses several chunks in one step
    s.upload()
    with pytest.raises(mg.MaviError) as e:
        mg.run_system(s, num_steps=2)
    assert e.value.status == mg.abi.MAVI_ERR_OUT_OF_GRID
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_jump_beyond_fixed_point_range(mg, precision):
    """A particle that moves more than two chunks within one step (8 length
    units against 3.05-unit chunks): the FP64 form steps on, as the reference
    does; the mixed form, whose fixed-point offsets reach 1.5 chunks from the
    centre of the chunk a particle is binned against, reports
    MAVI_ERR_OFFSET_RANGE instead of forming wrong pair terms."""
    s = lj_grid(mg, 8, 8, wall="periodic", chunks=(4, 4), precision=precision)
    s.calc_forces()
    s.state.vel[3] = (8000.0, 0.0)
    s.upload()
    if precision == "fp64":
        mg.run_system(s, num_steps=1)
        assert s.time_info.num_steps == 1
    else:
        with pytest.raises(mg.MaviError) as e:
            mg.run_system(s, num_steps=1)
        assert e.value.status == mg.abi.MAVI_ERR_OFFSET_RANGE
    s.close()


def test_outside_space_rejected_at_creation(mg):
    s = lj_grid(mg, 8, 8, wall="rigid", chunks=(4, 4))
    s.state.pos[0] = (-5.0, 1.0)
    with pytest.raises(mg.MaviError) as e:
        s.calc_forces()
    assert e.value.status == mg.abi.MAVI_ERR_OUTSIDE_SPACE


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_non_finite_position_reports_error(mg, precision):
    """A NaN position is turned into MAVI_ERR_NONFINITE by the binning's own
    check (the chunk index is clamped, no access leaves the arrays); the
    handle stays usable once the state is repaired."""
    s = lj_grid(mg, 8, 8, wall="periodic", chunks=(4, 4), precision=precision)
    s.calc_forces()
    good = s.state.pos[5].copy()
    s.state.pos[5] = (np.nan, 1.0)
    s.upload()
    with pytest.raises(mg.MaviError) as e:
        s.calc_forces()
    assert e.value.status == mg.abi.MAVI_ERR_NONFINITE
    s.state.pos[5] = good
    s.upload()
    s.calc_forces()
    s.close()


def test_injected_noise_missing_is_refused_before_any_launch(mg):
    s = self_propelled(mg, "szabo", noise="injected")
    h = s._ensure()
    assert h.lib.mavi_step(h.handle, 3) == mg.abi.MAVI_ERR_NOISE_MISSING
    s.run(1, noise=np.zeros(h.noise_count()))           # one step of noise: one step runs
    assert s.time_info.num_steps == 1
    s.close()


def test_chunk_overflow_reports_error(mg):
    s = soft_disks(mg, 256, phi=0.3)
    s.state.pos[:60] = s.state.pos[0]
    with pytest.raises(mg.MaviError) as e:
        s.calc_forces()
    assert e.value.status == mg.abi.MAVI_ERR_CHUNK_OVERFLOW


def test_profiling_events_inside_graph(mg):
    import ctypes as C
    s = lj_grid(mg, 20, 20, wall="periodic", use_graph=True)
    mg.run_system(s, num_steps=2)
    h = s.handle
    h.check(h.lib.mavi_profile_enable(h.handle, 1), "profile")
    h.step(3)
    p = mg.abi.MaviProfile()
    h.lib.mavi_profile_read(h.handle, C.byref(p))
    assert p.steps == 3 and p.step_ms > 0 and p.last_step_ms > 0
    assert p.launches[mg.abi.MAVI_KERNEL_FORCE] == 3
    assert p.ms[mg.abi.MAVI_KERNEL_FORCE] > 0
    h.check(h.lib.mavi_profile_enable(h.handle, 0), "profile off")
    h.step(2)
    s.close()


def test_overdamped_positions_only_state(mg, orc):
    """The overdamped step accepts a SecondLawState without velocities."""
    s = soft_disks(mg, 2048, precision="mixed")
    s.state.vel = None
    ref = orc.from_system(s, step_kind=mg.overdamped_step.kind)
    mg.run_system(s, num_steps=20, step_func=mg.overdamped_step)
    ref.step(20)
    assert np.max(np.abs(s.state.pos - ref.state()[0])) < 1e-4
    s.close()


def test_mixed_force_error_relaxed_packing(mg, orc):
    """Mixed-form force error on a relaxed soft-disk packing (forces small
    compared with the pair stiffness), normalised by the RMS force."""
    s = soft_disks(mg, 16384, precision="fp64")
    mg.run_system(s, num_steps=100, step_func=mg.overdamped_step)
    pos = s.state.pos.copy()
    s.close()
    m = soft_disks(mg, 16384, precision="mixed")
    m.state.pos[...] = pos
    ref = orc.from_system(m, step_kind=mg.overdamped_step.kind)
    err = rel_force_err(m.calc_forces(), ref.forces())
    assert err < MIXED_TOL, err
    m.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_staged_gather_equals_global_gather_bitwise(mg, precision):
    """The warp-staged shared-memory gather, the per-chunk global gather, the
    per-column gather and the autotuned choice sum the same terms in the same
    order. (The autotuner may take two or four lanes per particle for the
    soft disks, or the split gather for mixed Lennard-Jones, which sum in
    another order: then the results agree within 1e-6 of the RMS force, or
    1e-8 in position, instead.)"""
    out = []
    auto_mode = None
    for gather in ("staged", "global", "columns", "auto"):
        s = soft_disks(mg, 8192, precision=precision)
        s.int_cfg.device.gather = gather
        f = s.calc_forces()
        if gather == "auto":
            auto_mode = s.stats().gather_mode
        mg.run_system(s, num_steps=20, step_func=mg.overdamped_step)
        out.append((f, s.state.pos.copy()))
        s.close()
    for o in out[1:3]:
        assert np.array_equal(out[0][0], o[0])
        assert np.array_equal(out[0][1], o[1])
    if auto_mode in (0, 1, 2):
        assert np.array_equal(out[0][0], out[3][0]) and np.array_equal(out[0][1], out[3][1])
    else:
        assert precision == "mixed" and auto_mode in (5, 6)
        assert rel_force_err(out[3][0], out[0][0]) < 1e-6
    l = []
    for gather in ("staged", "global", "columns", "auto"):
        s = lj_grid(mg, 40, 40, wall="periodic", precision=precision)
        s.int_cfg.device.gather = gather
        mg.run_system(s, num_steps=20)
        l.append(s.state.pos.copy())
        if gather == "auto":
            auto_mode = s.stats().gather_mode
        s.close()
    for x in l[1:3]:
        assert np.array_equal(l[0], x)
    if auto_mode in (0, 1, 2):
        assert np.array_equal(l[0], l[3])
    else:   # the split gather (far pairs in FP32) sums in another order
        assert precision == "mixed" and auto_mode == 7
        assert np.max(np.abs(l[3] - l[0])) < 1e-8


def test_energy_drift_mixed_matches_fp64(mg):
    """Lennard-Jones gas (1024 particles, rigid box, dt = 1e-3, 2000 steps):
    the total energy of the mixed form follows the FP64 form's (same drift)."""
    series = {}
    for precision in ("fp64", "mixed"):
        s = lj_grid(mg, 32, 32, wall="rigid", chunks=(17, 17), precision=precision)
        e = []
        for _ in range(10):
            mg.run_system(s, num_steps=200)
            ke, pe = s.energies()
            e.append(ke + pe)
        series[precision] = np.array(e)
        s.close()
    e64, emx = series["fp64"], series["mixed"]
    scale = np.abs(e64).max()
    drift64 = abs(e64[-1] - e64[0]) / scale
    driftmx = abs(emx[-1] - emx[0]) / scale
    assert np.max(np.abs(emx - e64)) / scale < 1e-6
    assert abs(driftmx - drift64) < 1e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_periodic_circle_raw_displacement(mg, orc, precision):
    """Periodic walls on a circle: the stencil wraps but the reference takes
    the raw difference r1 - r2 (no minimum image) for wrapped neighbours."""
    from mavi_gb300 import workloads
    systems, step = workloads.lj_batch(num_replicas=2, precision=precision, n_min=1500, n_max=3000,
                                       quadrants=("periodic_circle",))
    b = mg.SystemBatch(systems, step)
    forces = b.calc_forces()
    for k, s in enumerate(systems):
        ref = orc.from_system(s, step_kind=step.kind)
        err = rel_force_err(forces[k], ref.forces())
        assert err < (FP64_TOL if precision == "fp64" else MIXED_TOL), (k, err)
        ref.close()
    b.run(50)
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("ntype", ["all", "rings"])
def test_rings_particle_neighbors_exact(mg, orc, precision, ntype):
    """Particle neighbour lists (src/rings/neighbors.jl:116-136): counts equal
    the oracle's and every list holds the same neighbours (order aside)."""
    from mavi_gb300 import rings as R, workloads
    systems, _ = workloads.rings_batch(num_replicas=1, rings_min=120, rings_max=120, precision=precision)
    s = systems[0]
    s.p_neighbors_cfg = R.NeighborsCfg(only_count=False, type=ntype, tol=1.1)
    s.run(300)                     # rings drift into contact
    s.calc_forces()                # a pair pass on the downloaded state
    counts, lists = s.neighbors()
    ref = orc.from_system(s)
    rc, rl = ref.rings_neighbors(tol=1.1, type_all=(ntype == "all"))
    assert np.array_equal(counts, rc)
    assert counts.sum() > 0
    for i in np.nonzero(counts)[0]:
        assert sorted(lists[i, :counts[i]]) == sorted(rl[i, :rc[i]])
        assert np.all(lists[i, counts[i]:] == -1)
    ref.close()
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rings_in_circular_container(mg, orc, precision):
    """Rings inside a PotentialWalls circle (no minimum image): the mixed form
    takes its ring geometry from the integer chunk offsets (exact shoelace
    area); forces and a 100-step trajectory with injected noise follow the
    oracle."""
    from mavi_gb300 import workloads
    systems, _ = workloads.rings_batch(num_replicas=1, rings_min=80, rings_max=80, precision=precision, k_bend=1.0)
    s = systems[0]
    s.int_cfg.device.noise = "injected"
    ref = orc.from_system(s)
    err = rel_force_err(s.calc_forces(), ref.forces())
    assert err < (FP64_TOL if precision == "fp64" else MIXED_TOL), err
    areas = ref.areas(s.state.num_rings)
    n = s.handle.noise_count()
    steps = 100
    noise = np.random.default_rng(5).normal(size=n * steps)
    s.run(steps, noise=noise)
    ref.step(steps, noise=noise)
    p, _, pol = ref.state()
    tol = 1e-8 if precision == "fp64" else 1e-3
    assert np.max(np.abs(s.state.pos - p)) < tol
    assert np.max(np.abs(s.state.pol - pol)) < tol
    assert np.all(areas > 0)
    ref.close()
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rings_container_wall_forces(mg, orc, precision):
    """Rings pressed against the PotentialWalls circle: calc_walls_forces!
    appears in the forces only when asked for (the step always includes it),
    and matches the oracle (the mixed form evaluates it in FP32 on the exact
    integer displacement from the centre)."""
    from mavi_gb300 import workloads
    systems, _ = workloads.rings_batch(num_replicas=1, rings_min=80, rings_max=80, precision=precision)
    s = systems[0]
    s.int_cfg.device.noise = "injected"
    st = s.state
    Rc = s.space_cfg.geometry_cfg.radius
    cms = st.rings_pos.mean(axis=1)
    # move the three outermost rings outwards until their outer particles sit
    # 0.1-0.3 inside the circle (the wall potential reaches 0.5 in)
    for q in np.argsort(-np.hypot(cms[:, 0], cms[:, 1]))[:3]:
        c = cms[q] / np.hypot(*cms[q])
        far = (st.rings_pos[q] @ c).max()
        st.rings_pos[q] += c * (Rc - 0.1 - 0.2 * (q % 2) - far)
    ref = orc.from_system(s)
    fw, f = s.calc_forces(include_walls=True), s.calc_forces(include_walls=False)
    rw, r = ref.forces(include_walls=True), ref.forces(include_walls=False)
    touched = np.hypot(*(rw - r).T) > 0
    assert touched.sum() >= 3
    assert np.array_equal(np.hypot(*(fw - f).T) > 0, touched)
    tol = FP64_TOL if precision == "fp64" else MIXED_TOL
    assert rel_force_err(f, r) < tol and rel_force_err(fw, rw) < tol
    # the wall term itself, against its own scale
    assert rel_force_err(fw - f, rw - r) < (1e-12 if precision == "fp64" else 1e-5)
    ref.close()
    s.close()


@pytest.mark.parametrize("kind,potential", [("slippery", None), ("potential", "harm"), ("potential", "lj")])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_line_walls(mg, orc, kind, potential, precision):
    """LinesCfg walls inside a rigid box: slippery segments (walls!,
    src/integration.jl:327-378) and PotentialWalls on segments
    (calc_walls_forces!, src/integration.jl:243-256, signed_pos
    src/configs.jl:119-135)."""
    from helpers import lj_lines
    s = lj_lines(mg, kind=kind, precision=precision, potential=potential or "harm")
    ref = orc.from_system(s)
    err = rel_force_err(s.calc_forces(include_walls=True), ref.forces(include_walls=True))
    assert err < (FP64_TOL if precision == "fp64" else MIXED_TOL), err
    mg.run_system(s, num_steps=1000)
    ref.step(1000)
    p, v, _ = ref.state()
    tol = 1e-8 if precision == "fp64" else 1e-3
    assert np.max(np.abs(s.state.pos - p)) < tol
    assert np.max(np.abs(s.state.vel - v)) < tol * 10
    s.close()


def test_resume_continues_the_device_noise(mg):
    """A system rebuilt from a snapshot (state + time_info) continues the
    device noise where the first run was (Philox counter = steps done), so the
    resumed trajectory equals the uninterrupted one bit for bit."""
    a = self_propelled(mg, "szabo", noise="device")
    a.run(20)
    pos, pol = a.state.pos.copy(), a.state.pol_angle.copy()
    ti = mg.system.TimeInfo(num_steps=a.time_info.num_steps, time=a.time_info.time)
    a.run(20)
    c = self_propelled(mg, "szabo", noise="device")
    c.state.pos[...] = pos
    c.state.pol_angle[...] = pol
    c.time_info = ti
    c.run(20)
    assert c.time_info.num_steps == a.time_info.num_steps == 40
    assert np.array_equal(c.state.pos, a.state.pos) and np.array_equal(c.state.pol_angle, a.state.pol_angle)
    a.close()
    c.close()


@pytest.mark.parametrize("gather", ["lanes2", "lanes4"])
def test_lanes_per_particle_soft_disks(mg, orc, gather):
    """Two or four lanes per particle (mixed soft disks, overdamped): forces
    within the mixed tolerance of the oracle and within 1e-6 of one lane per
    particle; the lanes' partial sums are combined in a fixed order, so two
    runs agree bit for bit."""
    runs = []
    for _ in range(2):
        s = soft_disks(mg, 16384, precision="mixed")
        s.int_cfg.device.gather = gather
        ref = orc.from_system(s, step_kind=mg.overdamped_step.kind)
        f = s.calc_forces()
        assert rel_force_err(f, ref.forces()) < MIXED_TOL
        assert s.stats().gather_mode == {"lanes2": 5, "lanes4": 6}[gather]
        mg.run_system(s, num_steps=30, step_func=mg.overdamped_step)
        runs.append((f, s.state.pos.copy()))
        ref.close()
        s.close()
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])
    one = soft_disks(mg, 16384, precision="mixed")
    one.int_cfg.device.gather = "columns"
    assert rel_force_err(runs[0][0], one.calc_forces()) < 1e-6
    one.close()


@pytest.mark.parametrize("gather", ["lanes2", "lanes4"])
def test_lanes_per_particle_szabo(mg, orc, gather):
    s = self_propelled(mg, "szabo", n=900, precision="mixed", noise="injected")
    s.int_cfg.device.gather = gather
    ref = orc.from_system(s)
    assert rel_force_err(s.calc_forces(), ref.forces()) < MIXED_TOL
    n = s._ensure().noise_count()
    noise = np.random.default_rng(4).normal(size=n * 30)
    s.run(30, noise=noise)
    ref.step(30, noise=noise)
    assert np.max(np.abs(s.state.pos - ref.state()[0])) < 1e-4
    s.close()


def test_lanes_reject_other_laws(mg):
    s = lj_grid(mg, 8, 8, precision="mixed")
    s.int_cfg.device.gather = "lanes2"
    with pytest.raises(mg.MaviError) as e:
        s.calc_forces()
    assert e.value.status == mg.abi.MAVI_ERR_UNSUPPORTED


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ragged_batch_with_tiny_replicas(mg, orc, precision):
    """Replicas of 1, 2, 3 and 6 particles beside a 400-particle one, rigid and
    periodic: chunk lists, forces and 50-step trajectories of every replica
    against the oracle (a lone particle has zero pair force)."""
    shapes = [(1, 1, "rigid"), (2, 1, "periodic"), (3, 1, "rigid"), (3, 2, "periodic"), (20, 20, "periodic")]
    systems = [lj_grid(mg, nx, ny, wall=w, precision=precision, seed=k) for k, (nx, ny, w) in enumerate(shapes)]
    b = mg.SystemBatch(systems)
    forces = b.calc_forces()
    refs = [orc.from_system(s) for s in systems]
    tol = FP64_TOL if precision == "fp64" else MIXED_TOL
    for k, (s, ref) in enumerate(zip(systems, refs)):
        assert chunks_equal_handle(b.handle.chunks(k), ref.chunks()), k
        fr = ref.forces()
        if k == 0:
            assert np.all(forces[k] == 0) and np.all(fr == 0)
        else:
            assert rel_force_err(forces[k], fr) < tol, k
    b.run(50)
    for k, (s, ref) in enumerate(zip(systems, refs)):
        ref.step(50)
        assert np.max(np.abs(s.state.pos - ref.state()[0])) < (1e-9 if precision == "fp64" else 1e-6), k
        ref.close()
    b.close()


def chunks_equal_handle(a, b):
    return np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_async_download_then_synchronize(mg):
    """mavi_download_state_async + mavi_synchronize give the arrays the
    blocking download gives; a device error of the queued work (a NaN position
    uploaded before the steps) is reported by mavi_synchronize."""
    import torch
    s = lj_grid(mg, 20, 20, wall="periodic")
    h = s._ensure()
    h.step(25)
    h.download()
    want_pos, want_vel = s.state.pos.copy(), s.state.vel.copy()
    pos = torch.zeros(want_pos.shape, dtype=torch.float64).pin_memory().numpy()
    vel = torch.zeros(want_vel.shape, dtype=torch.float64).pin_memory().numpy()
    h.download_async(pos, vel)
    h.synchronize()
    assert np.array_equal(pos, want_pos) and np.array_equal(vel, want_vel)
    bad = want_pos.copy()
    bad[7] = (np.nan, 1.0)
    h.check(h.lib.mavi_upload_state(h.handle, mg.abi.as_dptr(np.ascontiguousarray(bad)), None, None), "upload")
    h.step(1)
    h.download_async(pos, vel)
    with pytest.raises(mg.MaviError) as e:
        h.synchronize()
    assert e.value.status == mg.abi.MAVI_ERR_NONFINITE
    s.close()
