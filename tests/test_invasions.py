"""Invasion detection of the rings model (update_invasions! / check_invasions!,
src/rings/integration.jl:378-520; InvasionsCfg, src/rings/configs.jl:334-350).

CPU tests pin the oracle's restatement: a hand-made pair of rings with a known
answer, random configurations against an independent membership test
(winding numbers) and an independent transcription of the reference's
traversal order, chunked against all-pairs detection, the check schedule and
the all-pairs list that is never emptied. GPU tests compare the CUDA path's
lists, in order, with the oracle's."""
import ctypes as C

import numpy as np
import pytest

from helpers import rings_normal


# ---------------------------------------------------------------------------
# an independent point-in-polygon test and the reference's traversal order
# ---------------------------------------------------------------------------
def _winding_inside(p, poly):
    """Winding number of poly around p (nonzero: inside); agrees with the
    ray crossing parity of simple polygons away from edges and vertices."""
    w = 0
    n = len(poly)
    for i in range(n):
        a, b = poly[i], poly[(i + 1) % n]
        cross = (b[0] - a[0]) * (p[1] - a[1]) - (p[0] - a[0]) * (b[1] - a[1])
        if a[1] <= p[1] < b[1] and cross > 0:
            w += 1
        elif b[1] <= p[1] < a[1] and cross < 0:
            w -= 1
    return w != 0


def _find(rp, r1, r2, nmax, out, ns):
    for a, b in ((r1, r2), (r2, r1)):
        for i, p in enumerate(rp[a][:ns[a]]):
            if _winding_inside(p, rp[b][:ns[b]]):
                out.append((a + 1, b + 1, a * nmax + i + 1))


def _expected(rp, grid=None, bbox=None, ns=None):
    """check_invasions! with the winding-number membership: all pairs of ring
    ids, or the ring-chunk traversal (columns outer, rows inner, later rings
    of the chunk, then the neighbour chunks of an open grid)."""
    nr, nmax = rp.shape[0], rp.shape[1]
    ns = [nmax] * nr if ns is None else list(ns)
    out = []
    if grid is None:
        for r1 in range(nr):
            for r2 in range(r1 + 1, nr):
                _find(rp, r1, r2, nmax, out, ns)
        return out
    cols, rows = grid
    blx, bly, L, H = bbox
    cl, ch = L / cols, H / rows
    cms = np.stack([rp[r][:ns[r]].mean(axis=0) for r in range(nr)])
    lists = {}
    for r in range(nr):
        row = int((-cms[r, 1] + bly + H) // ch) + 1
        col = int((cms[r, 0] - blx) // cl) + 1
        lists.setdefault((row, col), []).append(r)

    def nbrs(i, j):
        if i == rows:
            return [(rows, j + 1)] if j < cols else []
        if j == 1:
            return [(i + 1, 1), (i + 1, 2), (i, 2)]
        if j == cols:
            return [(i + 1, cols - 1), (i + 1, cols)]
        return [(i + 1, j - 1), (i + 1, j), (i + 1, j + 1), (i, j + 1)]

    for col in range(1, cols + 1):
        for row in range(1, rows + 1):
            chunk = lists.get((row, col), [])
            for i, r1 in enumerate(chunk):
                for r2 in chunk[i + 1:]:
                    _find(rp, r1, r2, nmax, out, ns)
                for nb in nbrs(row, col):
                    for r2 in lists.get(nb, []):
                        _find(rp, r1, r2, nmax, out, ns)
    return out


def _ring(c, radius, n, phase):
    a = phase + 2 * np.pi * np.arange(n) / n
    return np.stack([c[0] + radius * np.cos(a), c[1] + radius * np.sin(a)], axis=1)


def _container(mg):
    """The circular container of the rings workloads (PotentialWalls inside)."""
    return mg.PotentialWalls(mg.HarmTruncCfg(k_rep=10.0, k_atr=0.0, dist_eq=0.5, dist_max=0.5), mode="inside")


def _system(mg, rings_pos, box=20.0, wall="container", invasions=None, r_chunks=None, precision="fp64"):
    """Rings in a PotentialWalls circle around the box [-box/2, box/2]^2 (its
    bounding box, _CIRCLE_BBOX for box 20, holds the ring chunks), or in the
    periodic box itself. Centred on the origin: construction's inside check
    ignores a circle's centre (src/space_checks.jl:53-60)."""
    R = mg.rings
    n = rings_pos.shape[1]
    inter = mg.HarmTruncCfg(k_rep=20.0, k_atr=4.0, dist_eq=1.0, dist_max=1.2)
    cfg = R.RingsCfg(p0=3.5, relax_time=1.0, vo=1.0, mobility=1.0, rot_diff=0.05, k_area=1.0, k_spring=20.0,
                     l_spring=1.0, num_particles=n, interaction_finder=inter)
    st = R.RingsState(rings_pos, np.zeros(rings_pos.shape[0]))
    if wall == "periodic":
        space = mg.SpaceCfg(mg.PeriodicWalls(), mg.RectangleCfg(box, box, (-box / 2, -box / 2)))
    else:
        space = mg.SpaceCfg(_container(mg), mg.CircleCfg(0.71 * box, (0.0, 0.0)))
    return R.RingsSystem(st, space, cfg,
                         R.RingsIntCfg(dt=0.001, r_chunks_cfg=r_chunks, invasions_cfg=invasions,
                                       device=mg.CUDADevice(precision=precision, noise="injected")))


_CIRCLE_BBOX = (-14.2, -14.2, 28.4, 28.4)


def _random_rings(seed, nr=30, n=12, box=20.0, radius=1.2):
    rng = np.random.default_rng(seed)
    c = rng.uniform(2.0 - box / 2, box / 2 - 2.0, size=(nr, 2))
    return np.stack([_ring(c[k], radius * rng.uniform(0.8, 1.2), n, rng.uniform(0, 2 * np.pi)) for k in range(nr)])


# ---------------------------------------------------------------------------
# oracle pins (no GPU)
# ---------------------------------------------------------------------------
def test_known_answer_two_rings(mg, orc):
    """Ring 1's vertex 0 reaches into ring 2, ring 2's vertex 3 into ring 1;
    find_invasions! pushes ring 1's points first."""
    n = 6
    r1 = _ring((-1.0, 0.0), 1.0, n, 0.1)
    r2 = _ring((0.75, 0.02), 1.0, n, 0.05)
    s = _system(mg, np.stack([r1, r2]), invasions=mg.rings.InvasionsCfg(0))
    o = orc.from_system(s)
    lst, last = o.rings_invasions()
    assert lst == [(1, 2, 1), (2, 1, n + 4)]
    assert last == 0


def test_golden_invasions_exact(mg, orc):
    """Known answers decided in exact rational arithmetic on dyadic vertices
    (tests/golden/make_golden.py): the oracle's FP64 list equals them."""
    import json
    from conftest import ROOT
    gold = json.loads((ROOT / "tests" / "golden" / "known_answers.json").read_text())["invasions"]
    assert len(gold) == 3
    for case in gold:
        rp = np.asarray(case["rings_pos"], dtype=np.float64)
        s = _system(mg, rp, invasions=mg.rings.InvasionsCfg(0))
        lst, _ = orc.from_system(s).rings_invasions()
        assert lst == [tuple(v) for v in case["invasions"]] and len(lst) > 0


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_rings_all_pairs(mg, orc, seed):
    rp = _random_rings(seed)
    s = _system(mg, rp, invasions=mg.rings.InvasionsCfg(0))
    lst, _ = orc.from_system(s).rings_invasions()
    exp = _expected(rp)
    assert lst == exp
    assert len(exp) > 10


@pytest.mark.parametrize("seed", [4, 5])
def test_random_rings_chunk_traversal(mg, orc, seed):
    rp = _random_rings(seed)
    s = _system(mg, rp, invasions=mg.rings.InvasionsCfg(0), r_chunks=mg.ChunksCfg(4, 3))
    lst, _ = orc.from_system(s).rings_invasions()
    assert lst == _expected(rp, grid=(4, 3), bbox=_CIRCLE_BBOX)
    # ring chunks wider than two ring radii find every invading pair
    s2 = _system(mg, rp, invasions=mg.rings.InvasionsCfg(0))
    full, _ = orc.from_system(s2).rings_invasions()
    assert sorted(lst) == sorted(full)


def _typed(mg, seed, nr=30, ns=(12, 7), box=20.0):
    """Two ring types of different sizes (rows past a ring's size are padding)."""
    R = mg.rings
    rng = np.random.default_rng(seed)
    types = rng.integers(1, 3, nr)
    c = rng.uniform(2.0 - box / 2, box / 2 - 2.0, size=(nr, 2))
    rp = np.zeros((nr, max(ns), 2))
    for k in range(nr):
        n = ns[types[k] - 1]
        rp[k, :n] = _ring(c[k], 1.2 * rng.uniform(0.8, 1.2), n, rng.uniform(0, 2 * np.pi))
        rp[k, n:] = rp[k, 0]
    inter = mg.HarmTruncCfg(k_rep=13.0, k_atr=0.1, dist_eq=1.0, dist_max=1.1)
    cfg = R.RingsCfg(p0=3.5, relax_time=1.0, vo=1.0, mobility=1.0, rot_diff=0.5, k_area=1.0, k_spring=20.0,
                     l_spring=[0.8, 0.8], num_particles=list(ns),
                     interaction_finder=R.InteractionMatrix([[inter, inter], [inter, inter]]))
    st = R.RingsState(rp, np.zeros(nr), num_particles=list(ns), types=list(types))
    space = mg.SpaceCfg(_container(mg), mg.CircleCfg(0.71 * box, (0.0, 0.0)))
    return rp, [ns[q - 1] for q in types], space, cfg, st


@pytest.mark.parametrize("chunks", [None, (4, 3)])
def test_two_ring_types(mg, orc, chunks):
    """Rings of two sizes: each polygon is its own type's points only, and
    p_id counts rows of nmax."""
    R = mg.rings
    rp, ns, space, cfg, st = _typed(mg, 11)
    rc = mg.ChunksCfg(*chunks) if chunks else None
    s = R.RingsSystem(st, space, cfg, R.RingsIntCfg(dt=0.001, r_chunks_cfg=rc, invasions_cfg=R.InvasionsCfg(0),
                                                    device=mg.CUDADevice(noise="injected")))
    lst, _ = orc.from_system(s).rings_invasions()
    exp = _expected(rp, grid=chunks, bbox=_CIRCLE_BBOX if chunks else None, ns=ns)
    assert lst == exp and len(exp) > 5


def test_check_schedule_and_last_check(mg, orc):
    rp = _random_rings(6)
    s = _system(mg, rp, invasions=mg.rings.InvasionsCfg(3), r_chunks=mg.ChunksCfg(4, 4))
    o = orc.from_system(s)
    assert o.rings_invasions() == ([], 0)          # construction: 0 - 0 < 3, no check
    rng = np.random.default_rng(0)
    seen = []
    for _ in range(8):
        o.step(1, orc.SEQUENTIAL, rng.standard_normal(o.noise_count()))
        seen.append(o.rings_invasions()[1])
    # checks at the start of the steps with num_steps 3 and 6
    assert seen == [0, 0, 0, 3, 3, 3, 6, 6]


def test_check_schedule_from_a_time_info(mg, orc):
    """A system constructed with a time_info: last_check starts at its
    num_steps (src/rings/rings.jl:276-278) and the checks follow from there."""
    rp = _random_rings(6)
    s = _system(mg, rp, invasions=mg.rings.InvasionsCfg(3), r_chunks=mg.ChunksCfg(4, 4))
    s.time_info = mg.system.TimeInfo(num_steps=100, time=1.0)
    o = orc.from_system(s)
    assert o.rings_invasions() == ([], 100)
    rng = np.random.default_rng(0)
    seen = []
    for _ in range(8):
        o.step(1, orc.SEQUENTIAL, rng.standard_normal(o.noise_count()))
        seen.append(o.rings_invasions()[1])
    assert seen == [100, 100, 100, 103, 103, 103, 106, 106]
    assert o.time()[0] == 108


def test_all_pairs_list_is_never_emptied(mg, orc):
    rp = _random_rings(7)
    s = _system(mg, rp, invasions=mg.rings.InvasionsCfg(1))
    o = orc.from_system(s)
    rng = np.random.default_rng(1)
    o.step(2, orc.SEQUENTIAL, rng.standard_normal(2 * o.noise_count()))
    first, last = o.rings_invasions()
    assert last == 1 and len(first) > 0
    o.step(1, orc.SEQUENTIAL, rng.standard_normal(o.noise_count()))
    second, last = o.rings_invasions()
    assert last == 2 and second[:len(first)] == first and len(second) > len(first)


def test_chunked_list_is_replaced(mg, orc):
    rp = _random_rings(8)
    s = _system(mg, rp, invasions=mg.rings.InvasionsCfg(0), r_chunks=mg.ChunksCfg(4, 4))
    o = orc.from_system(s)
    first, _ = o.rings_invasions()
    o.step(1, orc.SEQUENTIAL, np.zeros(o.noise_count()))
    second, last = o.rings_invasions()
    assert last == 0 and len(second) == len(first)   # steps_to_update 0: a check at every step start


def test_degenerate_ray_through_vertices_counts_nothing(mg, orc):
    """A point level with two vertices of the other ring: the strict
    inequalities of point_line_intersect see no crossing, so the reference
    (and both restatements) report no invasion there."""
    n = 6
    r1 = _ring((-1.0, 0.0), 1.0, n, 0.0)    # vertex 0 at (0, 0)
    r2 = _ring((0.8, 0.0), 1.0, n, 0.0)     # vertices 0 and 3 at y = 0
    s = _system(mg, np.stack([r1, r2]), invasions=mg.rings.InvasionsCfg(0))
    lst, _ = orc.from_system(s).rings_invasions()
    assert (1, 2, 1) not in lst


def test_invasions_abi_encoding(mg):
    R = mg.rings
    rp = _random_rings(9, nr=4)
    assert _system(mg, rp).invasions_abi() is None
    assert _system(mg, rp, invasions=R.InvasionsCfg(5)).invasions_abi() == (1, 5, 0, 0)
    assert _system(mg, rp, invasions=R.InvasionsCfg(2), r_chunks=mg.ChunksCfg(4, 3)).invasions_abi() == (1, 2, 4, 3)


def test_oracle_rejects_half_grid(mg, orc):
    rp = _random_rings(10, nr=4)
    s = _system(mg, rp)
    o = orc.from_system(s)
    with pytest.raises(RuntimeError):
        o.rings_invasions_config(1, 1, 3, 0)


# ---------------------------------------------------------------------------
# GPU parity
# ---------------------------------------------------------------------------
def _overlapped(mg, precision="fp64", wall="container", seed=3, **kw):
    """create_system_normal's 6 x 6 grid with the rings pushed into one
    another: towards the middle inside the circular container, randomly and
    wrapped when periodic (rings then straddle the boundary)."""
    s = _rings_normal(mg, precision=precision, wall=wall, **kw)
    st = s.state
    bb = s.space_cfg.bounding_box()
    bl = np.asarray(bb.bottom_left, dtype=float)
    size = np.array([bb.length, bb.height])
    cms = st.rings_pos.mean(axis=1, keepdims=True)
    if wall == "periodic":
        rng = np.random.default_rng(seed)
        shift = rng.uniform(-0.45, 0.45, size=(st.num_rings, 1, 2)) * 2.4
        st.rings_pos[...] = bl + np.mod(st.rings_pos + shift - bl, size)
    else:
        mid = bl + size / 2
        st.rings_pos[...] = (cms - mid) * 0.6 + mid + (st.rings_pos - cms)
    return s


def _rings_normal(mg, precision="fp64", wall="container", **kw):
    """create_system_normal's grid; unless periodic, inside the circular
    container inscribed in its rectangle."""
    s = rings_normal(mg, precision=precision, **kw)
    if wall == "container":
        g = s.space_cfg.geometry_cfg
        mid = np.array([g.bottom_left[0] + g.length / 2, g.bottom_left[1] + g.height / 2])
        s.state.rings_pos[...] -= mid                     # centred on the origin (see _system)
        s.space_cfg = mg.SpaceCfg(_container(mg), mg.CircleCfg(min(g.length, g.height) / 2, (0.0, 0.0)))
    return s


def _with_invasions(mg, s, steps, r_chunks):
    s.int_cfg.extra = mg.rings.IntCfgExtra(r_chunks, mg.rings.InvasionsCfg(steps))
    return s


def _gpu_list(s):
    info = s.invasions()
    return [(v.invasor, v.invaded, v.p_id) for v in info.list], info.last_check


@pytest.mark.gpu
@pytest.mark.parametrize("wall", ["container", "periodic"])
@pytest.mark.parametrize("chunks", [True, False])
def test_invasions_match_oracle_fp64(mg, orc, wall, chunks):
    s = _with_invasions(mg, _overlapped(mg, wall=wall), 2, mg.ChunksCfg(3, 3) if chunks else None)
    o = orc.from_system(s)
    assert _gpu_list(s) == o.rings_invasions()
    rng = np.random.default_rng(5)
    found = 0
    for _ in range(9):
        z = rng.standard_normal(o.noise_count())
        s.run(1, noise=z)
        o.step(1, orc.SEQUENTIAL, z)
        g = _gpu_list(s)
        assert g == o.rings_invasions()
        found = max(found, len(g[0]))
    assert found > 0
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("chunks", [True, False])
def test_invasions_mixed_form_on_the_same_state(mg, orc, chunks):
    """The mixed form moves the rings in FP32 steps; its check, in FP64 on
    the state it reached, equals the oracle's check of that state."""
    rc = mg.ChunksCfg(3, 3) if chunks else None
    s = _with_invasions(mg, _overlapped(mg, precision="mixed"), 5, rc)
    assert _gpu_list(s) == orc.from_system(s).rings_invasions() == ([], 0)
    nc = s._ensure().noise_count()
    rng = np.random.default_rng(8)
    found = 0
    acc = []                                              # without ring chunks the list is never emptied
    for k in (5, 4):                                      # checks at num_steps 5 and 10
        s.run(k, noise=rng.standard_normal(k * nc))      # no check inside: the state S at a check step
        snap = s.state.pos.copy()
        s.run(1, noise=rng.standard_normal(nc))           # this step checks S first
        ref = _with_invasions(mg, _rings_normal(mg), 0, rc)
        ref.state.pos[...] = snap
        lst, _ = orc.from_system(ref).rings_invasions()
        acc = lst if chunks else acc + lst
        g, last = _gpu_list(s)
        assert g == acc and last == s.time_info.num_steps - 1
        found = max(found, len(lst))
    assert found > 0
    s.close()


@pytest.mark.gpu
def test_invasions_with_sources_and_sinks(mg, orc):
    from test_sources import channel
    s = channel(mg)
    s.int_cfg.extra = mg.rings.IntCfgExtra(mg.ChunksCfg(3, 3), mg.rings.InvasionsCfg(5))
    o = orc.from_system(s)
    rng = np.random.default_rng(11)
    for _ in range(8):
        k = 25
        z = rng.standard_normal(o.noise_count() * k)
        z[36::37] = rng.random(k)
        s.run(k, noise=z)
        o.step(k, orc.SEQUENTIAL, z)
        assert _gpu_list(s) == o.rings_invasions()
    s.close()


@pytest.mark.gpu
def test_invasions_in_a_batch_of_replicas(mg, orc):
    a = _with_invasions(mg, _overlapped(mg, seed=3), 2, mg.ChunksCfg(3, 3))
    b = _with_invasions(mg, _overlapped(mg, wall="periodic", seed=4), 3, None)
    batch = mg.SystemBatch([a, b], device=mg.CUDADevice(precision="fp64", noise="injected"))
    oa, ob = orc.from_system(a), orc.from_system(b)
    nr = a.state.num_rings
    rng = np.random.default_rng(2)
    for _ in range(7):
        za, zb = rng.standard_normal(nr), rng.standard_normal(nr)
        batch.run(1, noise=np.concatenate([za, zb]))
        oa.step(1, orc.SEQUENTIAL, za)
        ob.step(1, orc.SEQUENTIAL, zb)
        assert _gpu_list(a) == oa.rings_invasions()
        assert _gpu_list(b) == ob.rings_invasions()
    # the other rings accessors read a batched system's own replica too
    for s_, o in ((a, oa), (b, ob)):
        ar, ra = s_.areas(), o.areas(nr)
        assert np.max(np.abs(ar - ra) / np.abs(ra)) < 1e-10
        mask, uids, na = s_.rings_ids()
        assert mask.all() and na == nr and np.array_equal(uids, np.arange(1, nr + 1))
    batch.close()


@pytest.mark.gpu
def test_invasions_config_errors(mg):
    s = _overlapped(mg)
    h = s._ensure()
    with pytest.raises(mg.abi.MaviError):
        h.check(h.lib.mavi_rings_invasions_config(h.handle, 0, 1, 1, 3, 0), "config")
    n, last = C.c_int64(), C.c_int64()
    h.check(h.lib.mavi_rings_invasions(h.handle, 0, None, 0, C.byref(n), C.byref(last)), "read")
    assert n.value == 0
    s.close()


@pytest.mark.gpu
def test_invasions_start_from_time_info(mg):
    """A system constructed with a time_info (e.g. a loaded one) keeps its step
    count on the device: last_check starts there and the schedule follows it."""
    s = _with_invasions(mg, _overlapped(mg), 3, mg.ChunksCfg(3, 3))
    s.time_info = mg.system.TimeInfo(num_steps=100, time=1.0)
    assert _gpu_list(s) == ([], 100)
    h = s._ensure()
    nc = h.noise_count()
    rng = np.random.default_rng(4)
    s.run(3, noise=rng.standard_normal(3 * nc))
    assert _gpu_list(s)[1] == 100                         # steps at num_steps 100..102 do not check
    s.run(1, noise=rng.standard_normal(nc))
    lst, last = _gpu_list(s)
    assert last == 103 and len(lst) > 0
    n, t = C.c_int64(), C.c_double()
    h.check(h.lib.mavi_get_time(h.handle, C.byref(n), C.byref(t)), "time")
    assert n.value == 104 == s.time_info.num_steps
    assert t.value == s.time_info.time
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("chunks", [None, (4, 3)])
def test_two_ring_types_gpu(mg, orc, chunks):
    R = mg.rings
    rp, ns, space, cfg, st = _typed(mg, 11)
    rc = mg.ChunksCfg(*chunks) if chunks else None
    s = R.RingsSystem(st, space, cfg, R.RingsIntCfg(dt=0.001, r_chunks_cfg=rc, invasions_cfg=R.InvasionsCfg(0),
                                                    device=mg.CUDADevice(noise="injected")))
    o = orc.from_system(s)
    assert _gpu_list(s) == o.rings_invasions()
    rng = np.random.default_rng(6)
    for _ in range(3):
        z = rng.standard_normal(o.noise_count())
        s.run(1, noise=z)
        o.step(1, orc.SEQUENTIAL, z)
        assert _gpu_list(s) == o.rings_invasions()
    s.close()


def _wrap(rp, box):
    return (rp + box / 2) % box - box / 2


def test_periodic_polygons_are_unwrapped_per_ring(mg, orc):
    """With periodic walls each ring's polygon is its continuous positions,
    unwrapped from its own first particle (update_continuos_pos!,
    src/rings/integration.jl:118-138), and no image of the other ring is
    taken: two rings that overlap across the boundary are in different frames
    and report nothing, while the same pair away from the boundary does."""
    n, box = 10, 20.0
    a = _ring((9.3, 0.05), 1.0, n, np.pi / 2)       # first particle at (9.3, 1.05): inside the box
    b = _ring((10.9, -0.02), 1.0, n, np.pi / 2 + 0.1)
    across = _wrap(np.stack([a, b]), box)           # b sits at the left edge, a straddles the right one
    inside = np.stack([a, b]) - np.array([5.0, 0.0])
    for rp, expect_none in ((across, True), (inside, False)):
        s = _system(mg, rp, box=box, wall="periodic", invasions=mg.rings.InvasionsCfg(0))
        lst, _ = orc.from_system(s).rings_invasions()
        if expect_none:
            assert lst == []
        else:
            assert lst == _expected(rp) and len(lst) > 0


@pytest.mark.gpu
def test_more_invasions_than_the_record_buffer(mg, orc):
    """36 rings stacked on one another: ~5,000 invasions in one check, more
    than the first record buffer holds; the buffer grows and the pairs are
    visited again, with the same list as the oracle's."""
    rng = np.random.default_rng(12)
    rp = np.stack([_ring(rng.uniform(-0.3, 0.3, 2), 1.0 + 0.1 * rng.random(), 10, rng.uniform(0, 2 * np.pi))
                   for _ in range(36)])
    s = _system(mg, rp, invasions=mg.rings.InvasionsCfg(0))
    lst, last = orc.from_system(s).rings_invasions()
    assert len(lst) > 1024
    assert _gpu_list(s) == (lst, last)
    s.close()


@pytest.mark.gpu
def test_golden_invasions_exact_gpu(mg):
    """The CUDA check against the exact known answers, with and without ring
    chunks (one 4 x 4 grid holds every pair as neighbours here)."""
    import json
    from conftest import ROOT
    gold = json.loads((ROOT / "tests" / "golden" / "known_answers.json").read_text())["invasions"]
    for case in gold:
        rp = np.asarray(case["rings_pos"], dtype=np.float64)
        want = [tuple(v) for v in case["invasions"]]
        s = _system(mg, rp, invasions=mg.rings.InvasionsCfg(0))
        assert _gpu_list(s) == (want, 0)
        s.close()
        s = _system(mg, rp, invasions=mg.rings.InvasionsCfg(0), r_chunks=mg.ChunksCfg(4, 4))
        assert sorted(_gpu_list(s)[0]) == sorted(want)
        s.close()
