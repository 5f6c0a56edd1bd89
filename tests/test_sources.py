"""Variable number of rings with sources and sinks (VarRingsIds,
src/rings/states.jl:20-40, 152-223; src/rings/sources.jl; step! head
src/rings/integration.jl:522-526).

CPU tests pin the oracle's restatement on hand-made cases, including the
reference's quirks (the active-id view of a second sink, chunk lists that end
early at the grid's last row); GPU tests compare the CUDA path with the oracle
over hundreds of steps with sinks and sources firing."""
import numpy as np
import pytest

from helpers import rings_normal


def _grid(s):
    bb = s.space_cfg.bounding_box()
    cc = s.int_cfg.chunks_cfg
    return (float(bb.bottom_left[0]), float(bb.bottom_left[1]), float(bb.length), float(bb.height),
            int(cc.num_rows), int(cc.num_cols))


def _box_around(R, tpl, pad, pol=0.0, size=(1, 1), offset=(0.0, 0.0)):
    """A source whose first box spawns exactly at the template's place."""
    return R.SourceCfg(bottom_left=(tpl[:, 0].min() - pad, tpl[:, 1].min() - pad), spawn_pos=tpl.copy(),
                       spawn_pol=pol, pad=pad, size=size, offset=offset)


def channel(mg, precision="fp64", random_pol=True, use_chunks=True):
    """36 rings drifting to +x in a periodic box; the middle column starts
    inactive, two sources spawn where its rings were, a sink spans the right
    column."""
    R = mg.rings
    s = rings_normal(mg, precision=precision, use_chunks=use_chunks)
    st = s.state
    st.pol[:] = 0.0
    mask = np.ones(st.num_rings, bool)
    mask[12:18] = False
    st.active_state = R.ActiveState(mask)
    src = _box_around(R, st.rings_pos[14], 0.05)
    src2 = _box_around(R, st.rings_pos[15], 0.05, pol="random" if random_pol else 0.3)
    cms = st.rings_pos.mean(axis=1)
    x5 = cms[30:36, 0].mean()
    g = s.space_cfg.geometry_cfg
    sink = R.SinkCfg(mg.RectangleCfg(1.0, g.height, (x5 - 0.5, g.bottom_left[1])))
    s.source_cfg = [sink, src, src2]
    return s


# ---------------------------------------------------------------------------
# host computation of Source(...) (src/rings/sources.jl:122-185)
# ---------------------------------------------------------------------------
def test_source_boxes_grid_and_spawn_points(mg):
    R = mg.rings
    tpl = np.array([[1.0, 2.0], [2.0, 2.5], [1.5, 3.0]])
    cfg = R.SourceCfg(bottom_left=(10.0, 20.0), spawn_pos=tpl, pad=0.1, offset=(0.5, 0.25), size=(2, 3))
    boxes, spawns, lists = R.source_boxes(cfg)
    assert lists is None
    L, H = (2.0 - 1.0) + 2 * 0.1, (3.0 - 2.0) + 2 * 0.1
    k = 0
    for i in range(1, 3):
        for j in range(1, 4):
            bx, by = 10.0 + ((i - 1) * L + i * 0.5), 20.0 + ((j - 1) * H + j * 0.25)
            assert boxes[k] == (bx, by, L, H)
            # the template's lower-left corner sits pad inside the box
            assert np.array_equal(spawns[k], tpl + np.array([bx - 1.0 + 0.1, by - 2.0 + 0.1]))
            k += 1


def test_chunk_lists_are_the_intersecting_chunks(mg):
    R = mg.rings
    s = channel(mg)
    grid = _grid(s)
    gblx, gbly, glen, ghei, rows, cols = grid
    cl, ch = glen / cols, ghei / rows
    for c in s.source_cfg[1:]:
        boxes, _, lists = R.source_boxes(c, grid)
        pad = c.pad
        for b, lst in zip(boxes, lists):
            bp = (b[0] - pad, b[1] - pad, b[2] + 2 * pad, b[3] + 2 * pad)
            brute = {(r - 1, q - 1) for q in range(1, cols + 1) for r in range(1, rows + 1)
                     if R._intersects((gblx + (q - 1) * cl, gbly + ghei - r * ch, cl, ch), bp)}
            assert lst and set(lst) == brute


def test_chunk_list_empty_when_box_reaches_last_row(mg):
    """ChunksChecker's row loop ends its range only at a row below the box:
    a box reaching the grid's bottom row gets no chunks, so it always reads as
    empty (src/rings/sources.jl:85-100)."""
    R = mg.rings
    s = rings_normal(mg)
    tpl = s.state.rings_pos[0]          # the bottom-left ring
    _, _, lists = R.source_boxes(_box_around(R, tpl, 0.05), _grid(s))
    assert lists == [[]]


# ---------------------------------------------------------------------------
# oracle semantics
# ---------------------------------------------------------------------------
def _noise(o, k, seed=7):
    return np.random.default_rng(seed).standard_normal(o.noise_count() * k)


def test_first_step_removes_sink_rings_and_spawns(mg, orc):
    s = channel(mg, random_pol=False)
    st = s.state
    cms0 = st.rings_pos.mean(axis=1)
    o = orc.from_system(s)
    m, u, na = o.rings_ids()
    assert na == 30 and not m[12:18].any() and np.array_equal(u, np.arange(1, 37))
    z = _noise(o, 1)
    z[:36] = 0.0                       # no rotational noise: the spawn angles stay within 0.02
    o.step(1, orc.SEQUENTIAL, z)
    m, u, na = o.rings_ids()
    sink = s.source_cfg[0].geometry_cfg
    inside = (cms0[:, 0] >= sink.bottom_left[0]) & (cms0[:, 0] <= sink.bottom_left[0] + sink.length)
    assert inside[30:36].all() and not inside[:30].any()
    # the sink removed column 5; the two sources filled the first free slots (12, 13)
    expect = np.ones(36, bool)
    expect[14:18] = False
    expect[30:36] = False
    assert np.array_equal(m, expect) and na == 26
    assert u[12] == 37 and u[13] == 38
    pos, _, pol = o.state()
    assert abs(pol[12] - 0.0) < 0.02 and abs(pol[13] - 0.3) < 0.02
    # spawned at the templates, then moved by one step
    assert np.max(np.abs(pos.reshape(36, 10, 2)[12] - st.rings_pos[14])) < 0.05
    # removed rings keep their positions
    assert np.array_equal(pos.reshape(36, 10, 2)[30:36], st.rings_pos[30:36])


def test_second_sink_sees_a_shortened_view(mg, orc):
    """process_sink! iterates ids[1:num_active] and remove_ring! decrements
    num_active: a second sink in the same step does not reach the last ids."""
    R = mg.rings
    s = rings_normal(mg)
    st = s.state
    cms = st.rings_pos.mean(axis=1)
    g = s.space_cfg.geometry_cfg

    def column_sink(c):
        x = cms[6 * c:6 * c + 6, 0].mean()
        return R.SinkCfg(mg.RectangleCfg(1.0, g.height, (x - 0.5, g.bottom_left[1])))

    st.active_state = R.ActiveState(True)
    s.source_cfg = [column_sink(0), column_sink(5)]
    o = orc.from_system(s)
    o.step(1, orc.SEQUENTIAL, _noise(o, 1))
    m, _, na = o.rings_ids()
    # sink 1 removed rings 0-5; sink 2's view ids[1:30] stopped at ring 29
    assert not m[0:6].any() and m[6:36].all() and na == 30
    o.step(1, orc.SEQUENTIAL, _noise(o, 1, 8))
    m, _, na = o.rings_ids()
    assert not m[30:36].any() and na == 24


def test_random_spawn_polarisation_uses_the_step_uniform(mg, orc):
    s = channel(mg, random_pol=True)
    o = orc.from_system(s)
    assert o.noise_count() == 36 + 1
    z = _noise(o, 1)
    z[:36] = 0.0
    z[36] = 0.25
    o.step(1, orc.SEQUENTIAL, z)
    pol = o.state()[2]
    assert abs(pol[13] - 0.25 * 2.0 * 3.141592653589793) < 0.02


def test_no_free_slot_adds_nothing(mg, orc):
    R = mg.rings
    s = rings_normal(mg)
    st = s.state
    # a box at the bottom row reads as empty (no chunk list), but every slot is taken
    s.source_cfg = [_box_around(R, st.rings_pos[0], 0.05)]
    st.active_state = R.ActiveState(True)
    o = orc.from_system(s)
    o.step(3, orc.SEQUENTIAL, _noise(o, 3))
    m, u, na = o.rings_ids()
    assert m.all() and na == 36 and np.array_equal(u, np.arange(1, 37))


def test_inactive_rings_take_no_part(mg, orc):
    """An ActiveState alone: inactive rings neither move nor push."""
    R = mg.rings
    s = rings_normal(mg)
    mask = np.ones(36, bool)
    mask[::2] = False
    s.state.active_state = R.ActiveState(mask)
    o = orc.from_system(s)
    f = o.forces()
    assert np.all(f.reshape(36, 10, 2)[::2] == 0.0)
    o.step(5, orc.SEQUENTIAL, _noise(o, 5))
    pos = o.state()[0].reshape(36, 10, 2)
    assert np.array_equal(pos[::2], s.state.rings_pos[::2])
    assert not np.array_equal(pos[1::2], s.state.rings_pos[1::2])


# ---------------------------------------------------------------------------
# GPU parity
# ---------------------------------------------------------------------------
def _compare(s, o, tol):
    m, u, na = s.rings_ids()
    mo, uo, nao = o.rings_ids()
    assert np.array_equal(m, mo) and np.array_equal(u, uo) and na == nao
    pos, _, pol = o.state()
    assert np.max(np.abs(s.state.pos - pos)) <= tol
    assert np.max(np.abs(s.state.pol - pol)) <= tol
    return na, u.max()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sources_sinks_match_oracle(mg, orc, precision):
    s = channel(mg, precision=precision)
    o = orc.from_system(s)
    _compare(s, o, 0.0)
    f = s.calc_forces()
    assert np.all(f.reshape(36, 10, 2)[12:18] == 0.0)
    rng = np.random.default_rng(11)
    k, rounds = 100, (12 if precision == "fp64" else 6)
    events = set()
    for _ in range(rounds):
        z = rng.standard_normal(o.noise_count() * k)
        z[36::37] = rng.random(k)      # the spawn box's uniforms
        s.run(k, noise=z)
        o.step(k, orc.SEQUENTIAL, z)
        events.add(_compare(s, o, 1e-8 if precision == "fp64" else 1e-3))
    assert len(events) >= (3 if precision == "fp64" else 2)   # removals and spawns along the way


@pytest.mark.gpu
def test_sources_without_chunks_use_all_particles(mg, orc):
    s = channel(mg, use_chunks=False, random_pol=False)
    o = orc.from_system(s)
    rng = np.random.default_rng(12)
    for _ in range(3):
        z = rng.standard_normal(o.noise_count() * 50)
        s.run(50, noise=z)
        o.step(50, orc.SEQUENTIAL, z)
        _compare(s, o, 1e-8)


@pytest.mark.gpu
def test_active_state_only_matches_oracle(mg, orc):
    R = mg.rings
    s = rings_normal(mg)
    mask = np.ones(36, bool)
    mask[::3] = False
    s.state.active_state = R.ActiveState(mask)
    o = orc.from_system(s)
    p0 = s.state.rings_pos.copy()
    z = np.random.default_rng(13).standard_normal(o.noise_count() * 200)
    s.run(200, noise=z)
    o.step(200, orc.SEQUENTIAL, z)
    _compare(s, o, 1e-8)
    pos = s.state.pos.reshape(36, 10, 2)
    assert np.array_equal(pos[::3], p0[::3])
    assert not np.array_equal(pos[1::3], p0[1::3])


@pytest.mark.gpu
def test_sources_with_device_noise_run(mg):
    s = channel(mg, precision="mixed")
    s.int_cfg.device.noise = "device"
    s.run(300)
    m, u, na = s.rings_ids()
    assert na >= 20 and u.max() >= 38 and m.sum() == na


@pytest.mark.gpu
def test_experiment_checkpoint_keeps_the_active_rings(mg, tmp_path):
    """A checkpoint of a system with sources and sinks keeps which rings are
    active; a resumed run starts from that mask."""
    ex = mg.experiments
    s = channel(mg, random_pol=False)
    s.int_cfg.device.noise = "device"
    exp = ex.Experiment(ex.ExperimentCfg(tf=2.0, root=str(tmp_path / "a"), checkpoint_cfg=ex.CheckpointCfg(1.0)),
                        ex.DelayedCfg(0.5), s)
    ex.run_experiment(exp)
    s.close()
    s2 = channel(mg, random_pol=False)
    s2.int_cfg.device.noise = "device"
    ex.load_experiment(tmp_path / "a", s2, ex.DelayedCfg(0.5))
    import json
    info = json.loads((tmp_path / "a" / "checkpoint" / "checkpoint_info.json").read_text())
    saved = np.load(tmp_path / "a" / "checkpoint" / info["last_used"] / "sys_state" / "state.npz")["active_mask"]
    m, _, na = s2.rings_ids()
    assert np.array_equal(m, saved.astype(bool)) and na == int(saved.sum())
    assert not m[30:36].any()            # the sink had removed the right column
    s2.close()


@pytest.mark.gpu
def test_sources_in_a_batch_of_replicas(mg, orc):
    """Two replicas with sources and sinks in one handle: each replica's head
    of step runs in its own block; the step's noise holds every replica's
    ring normals first, then every replica's spawn uniforms."""
    a = channel(mg, random_pol=True)
    b = channel(mg, random_pol=True)
    b.state.pol[:] = 0.4                                     # the second replica drifts another way
    batch = mg.SystemBatch([a, b], device=mg.CUDADevice(precision="fp64", noise="injected"))
    oa, ob = orc.from_system(a), orc.from_system(b)
    nr = a.state.num_rings
    rng = np.random.default_rng(21)
    for _ in range(4):
        k = 100
        za = rng.standard_normal((k, nr + 1))
        zb = rng.standard_normal((k, nr + 1))
        za[:, nr] = rng.random(k)
        zb[:, nr] = rng.random(k)
        # batch layout per step: [a rings][b rings][a spawn][b spawn]
        z = np.concatenate([za[:, :nr], zb[:, :nr], za[:, nr:], zb[:, nr:]], axis=1).reshape(-1)
        batch.run(k, noise=z)
        oa.step(k, orc.SEQUENTIAL, za.reshape(-1))
        ob.step(k, orc.SEQUENTIAL, zb.reshape(-1))
        for s_, o in ((a, oa), (b, ob)):
            pos, _, pol = o.state()
            assert np.max(np.abs(s_.state.pos - pos)) < 1e-8
            assert np.max(np.abs(s_.state.pol - pol)) < 1e-8
    h = batch.handle
    import ctypes as C
    for r, o in enumerate((oa, ob)):
        m = np.zeros(nr, dtype=np.int32)
        u = np.zeros(nr, dtype=np.int32)
        na = C.c_int32()
        h.check(h.lib.mavi_rings_active(h.handle, r, mg.abi.as_iptr(m), mg.abi.as_iptr(u), C.byref(na)), "active")
        mo, uo, nao = o.rings_ids()
        assert np.array_equal(m.astype(bool), mo) and np.array_equal(u, uo) and na.value == nao
    batch.close()


# ---------------------------------------------------------------------------
# host encoding for mavi_rings_sources (no GPU)
# ---------------------------------------------------------------------------
def test_sources_abi_encoding(mg, orc):
    R = mg.rings
    s = channel(mg, random_pol=True)
    s.source_cfg.append(R.SinkCfg(mg.CircleCfg(2.0, (5.0, 6.0))))
    mask, n, entries, boxes, spawn_xy, chunk_rc = s.sources_abi()
    abi = mg.abi
    assert n == 4 and mask.dtype == np.int32 and mask.sum() == 30
    kinds = [entries[k].kind for k in range(n)]
    assert kinds == [abi.MAVI_SRC_SINK, abi.MAVI_SRC_SOURCE, abi.MAVI_SRC_SOURCE, abi.MAVI_SRC_SINK]
    assert entries[0].geometry == abi.MAVI_GEOM_RECTANGLE and entries[3].geometry == abi.MAVI_GEOM_CIRCLE
    assert (entries[3].radius, entries[3].cx, entries[3].cy) == (2.0, 5.0, 6.0)
    assert entries[1].pol_mode == abi.MAVI_SPAWN_POL_FIXED and entries[2].pol_mode == abi.MAVI_SPAWN_POL_RANDOM
    assert entries[1].num_boxes == 1 and entries[2].num_boxes == 1
    # one spawn template of nmax points per box, the boxes' chunk lists concatenated
    assert spawn_xy.size == 2 * 2 * s.state.nmax
    assert chunk_rc.size == 2 * (boxes[0].num_chunks + boxes[1].num_chunks)
    # the oracle takes the same encoding; its step noise grows by the random box
    o = orc.from_system(s)
    assert o.noise_count() == s.state.num_rings + 1


def test_sources_reject_bad_configuration(mg):
    R = mg.rings
    s = rings_normal(mg)
    with pytest.raises(ValueError):
        R.RingsSystem(s.state, s.space_cfg, s.dynamic_cfg, s.int_cfg,
                      source_cfg=R.SourceCfg(bottom_left=(0.0, 0.0), spawn_pos=np.zeros((3, 2))))
    with pytest.raises(ValueError):
        R.RingsSystem(s.state, s.space_cfg, s.dynamic_cfg, s.int_cfg, source_cfg="not a source")
    with pytest.raises(ValueError):
        R.ActiveState(np.ones(5, bool)).get_active_mask(36)
    bad = rings_normal(mg)
    bad.source_cfg = [R.SourceCfg(bottom_left=(1.0, 1.0), spawn_pos=bad.state.rings_pos[14].copy(), spawn_pol="spin")]
    with pytest.raises(ValueError):
        bad.sources_abi()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sources_in_the_circular_container(mg, orc, precision):
    """Sources and sinks with the PotentialWalls circle of the rings workloads
    (no minimum image; the mixed form's integer ring geometry and FP32 wall
    force) and a quarter of the rings parked at the start."""
    from mavi_gb300 import workloads
    R = mg.rings
    systems, _ = workloads.rings_batch(num_replicas=1, rings_min=80, rings_max=80, precision=precision)
    s = systems[0]
    s.int_cfg.device.noise = "injected"
    st = s.state
    nr = st.num_rings
    cms = st.rings_pos.mean(axis=1)
    mask = np.ones(nr, bool)
    mask[::4] = False
    st.active_state = R.ActiveState(mask)
    q = int(np.argmin(np.hypot(cms[:, 0], cms[:, 1])))          # the most central ring, parked
    mask[q] = False
    tpl = st.rings_pos[q]
    pad = 0.05
    src = R.SourceCfg(bottom_left=(tpl[:, 0].min() - pad, tpl[:, 1].min() - pad), spawn_pos=tpl.copy(),
                      spawn_pol=0.7, pad=pad)
    far = int(np.argmax(cms[:, 0]))
    sink = R.SinkCfg(mg.CircleCfg(6.0, (float(cms[far, 0]), float(cms[far, 1]))))
    s.source_cfg = [src, sink]
    o = orc.from_system(s)
    rng = np.random.default_rng(31)
    tol = 1e-8 if precision == "fp64" else 1e-3
    for _ in range(2):
        z = rng.standard_normal(o.noise_count() * 100)
        s.run(100, noise=z)
        o.step(100, orc.SEQUENTIAL, z)
        m, u, na = s.rings_ids()
        mo, uo, nao = o.rings_ids()
        assert np.array_equal(m, mo) and np.array_equal(u, uo) and na == nao
        pos, _, pol = o.state()
        real = np.array([k % st.nmax < st.ring_num_particles(k // st.nmax) for k in range(s.num_slots)])
        assert np.max(np.abs(s.state.pos[real] - pos[real])) < tol
        assert np.max(np.abs(s.state.pol - pol)) < tol
    assert u.max() > nr                   # the source spawned
    assert not m[far]                     # the sink removed the ring it covers
    o.close()
    s.close()
