"""Pins the oracle (the CPU FP64 restatement of the reference) against
closed-form known answers (tests/golden/known_answers.json, generated with
exact arithmetic by tests/golden/make_golden.py) and against the reference's
own self-consistency tests (test/tests_rings/tests_general.jl:16-45):
chunked == all-pairs and threaded == sequential."""
import json
import math

import numpy as np
import pytest

from conftest import ROOT

GOLD = json.loads((ROOT / "tests" / "golden" / "known_answers.json").read_text())


def test_julia_div_matches_exact_truncated_quotient(orc):
    # compared by value: the sign of a zero quotient is irrelevant because
    # update_particle_chunk! applies trunc(Int, .) to it (src/chunks.jl:129-130)
    for c in GOLD["julia_div"]:
        got = orc.julia_div(c["x"], c["y"])
        assert got == c["div"], c


def _params(mg, n, space, dyn, chunks, step=0, dt=1e-3):
    from mavi_gb300 import abi
    p = abi.MaviReplicaParams()
    p.num_particles = n
    p.state_kind = abi.MAVI_STATE_SECOND_LAW
    p.step_kind = step
    p.dt = dt
    if chunks:
        p.chunk_cols, p.chunk_rows = chunks
    space.fill(p)
    dyn.fill(p.dyn)
    return p


def test_chunk_index_known_answers(mg, orc):
    g = GOLD["chunk_grid"]
    geom = mg.RectangleCfg(g["length"], g["height"], tuple(g["bl"]))
    p = _params(mg, 1, mg.SpaceCfg(mg.RigidWalls(), geom), mg.HarmTruncCfg(1, 0, 0.1, 0.1), (g["cols"], g["rows"]))
    o = orc.OracleSystem(p, np.array([[0.0, 5.0]]), np.zeros((1, 2)))
    for c in GOLD["chunk_index"]:
        st, row, col = o.chunk_of(c["x"], c["y"])
        assert st == 0 and (row, col) == (c["row"], c["col"]), c


def test_out_of_grid_raises_like_bounds_error(mg, orc):
    geom = mg.RectangleCfg(10.0, 10.0)
    p = _params(mg, 2, mg.SpaceCfg(mg.RigidWalls(), geom), mg.HarmTruncCfg(1, 0, 1, 1), (5, 5))
    o = orc.OracleSystem(p, np.array([[1.0, 1.0], [5.0, 5.0]]), np.zeros((2, 2)))
    assert o.status == 0
    o.set_state(np.array([[-2.5, 1.0], [5.0, 5.0]]), np.zeros((2, 2)))
    assert o.update_chunks() == 3  # MAVI_ERR_OUT_OF_GRID


def test_chunk_overflow_raises(mg, orc):
    geom = mg.RectangleCfg(10.0, 10.0)
    # chunk 5 x 5 with radius 0.5: capacity 2*(5+1)^2 = 72 (src/chunks.jl:32-34)
    p = _params(mg, 80, mg.SpaceCfg(mg.RigidWalls(), geom), mg.HarmTruncCfg(1, 0, 1.0, 1.0), (2, 2))
    pos = np.full((80, 2), 1.0)
    o = orc.OracleSystem(p, pos, np.zeros((80, 2)))
    assert o.status == 4  # MAVI_ERR_CHUNK_OVERFLOW


def test_capacity_known_answers(mg):
    for c in GOLD["capacity"]:
        assert mg.chunk_capacity(c["chunk_l"], c["chunk_l"], c["r"]) == c["cap"]


def test_rectangular_grid_known_answer(mg):
    g = GOLD["grid"]
    pos, geom = mg.rectangular_grid(g["nx"], g["ny"], g["offset"], g["radius"])
    assert pos.shape == (g["nx"] * g["ny"], 2)
    assert pos[0, 0] == g["first"][0] and pos[0, 1] == g["first"][1]
    assert geom.length == g["length"]


def _two_particle_force(mg, orc, dyn, d):
    geom = mg.RectangleCfg(100.0, 100.0)
    p = _params(mg, 2, mg.SpaceCfg(mg.RigidWalls(), geom), dyn, None)
    pos = np.array([[40.0, 50.0], [40.0 + d, 50.0]])
    o = orc.OracleSystem(p, pos, np.zeros((2, 2)))
    return o.forces()


def test_pair_force_known_answers(mg, orc):
    for c in GOLD["lj_pair"]:
        f = _two_particle_force(mg, orc, mg.LenJonesCfg(c["sigma"], c["epsilon"]), c["d"])
        assert f[1, 0] == pytest.approx(c["force_on_right"], rel=1e-13, abs=1e-13)
        assert f[0, 0] == -f[1, 0] and f[0, 1] == 0
    for c in GOLD["harm_pair"]:
        f = _two_particle_force(mg, orc, mg.HarmTruncCfg(c["k_rep"], c["k_atr"], c["dist_eq"], c["dist_max"]), c["d"])
        assert f[1, 0] == pytest.approx(c["force_on_right"], rel=1e-13, abs=1e-13)


def test_periodic_stencil_matches_reference_definition(mg, orc):
    """get_neighbors(…, ::PeriodicWalls) restated independently (src/chunks.jl:61-87)."""
    geom = mg.RectangleCfg(12.0, 8.0)
    rows, cols = 4, 6
    p = _params(mg, 1, mg.SpaceCfg(mg.PeriodicWalls(), geom), mg.HarmTruncCfg(1, 0, 1, 1), (cols, rows))
    o = orc.OracleSystem(p, np.array([[1.0, 1.0]]), np.zeros((1, 2)))
    cnt, nb = o.neighbors()

    def get_id(x, n):
        return n if x == 0 else (1 if x % (n + 1) == 0 else x)
    for i in range(1, rows + 1):
        for j in range(1, cols + 1):
            want = [(get_id(i + 1, rows), get_id(j, cols)), (get_id(i + 1, rows), get_id(j + 1, cols)),
                    (get_id(i, rows), get_id(j + 1, cols)), (get_id(i - 1, rows), get_id(j + 1, cols))]
            c = (j - 1) * rows + (i - 1)
            got = [(int(x) % rows + 1, int(x) // rows + 1) for x in nb[c, :cnt[c]]]
            assert got == want


def test_open_stencil_is_clipped_half_shell(mg, orc):
    """get_neighbors for open walls (src/chunks.jl:89-118)."""
    geom = mg.RectangleCfg(12.0, 8.0)
    rows, cols = 4, 6
    p = _params(mg, 1, mg.SpaceCfg(mg.RigidWalls(), geom), mg.HarmTruncCfg(1, 0, 1, 1), (cols, rows))
    o = orc.OracleSystem(p, np.array([[1.0, 1.0]]), np.zeros((1, 2)))
    cnt, nb = o.neighbors()
    pairs = set()
    for c in range(rows * cols):
        for x in nb[c, :cnt[c]]:
            pairs.add(frozenset((c, int(x))))
    # every 8-neighbour pair of the grid exactly once, nothing else
    want = set()
    for c in range(rows * cols):
        i, j = c % rows, c // rows
        for di in (-1, 0, 1):
            for dj in (-1, 0, 1):
                if (di, dj) != (0, 0) and 0 <= i + di < rows and 0 <= j + dj < cols:
                    want.add(frozenset((c, (j + dj) * rows + i + di)))
    assert pairs == want
    assert int(cnt.sum()) == len(want)


def _harm_system(mg, n, wall, seed, chunks=(12, 12), L=24.0):
    rng = np.random.default_rng(seed)
    pos = rng.random((n, 2)) * L
    vel = rng.normal(0, 0.3, (n, 2))
    dyn = mg.HarmTruncCfg(k_rep=20.0, k_atr=4.0, dist_eq=1.0, dist_max=1.2)
    return mg.System(mg.SecondLawState(pos, vel), mg.SpaceCfg(wall, mg.RectangleCfg(L, L)), dyn,
                     mg.IntCfg(dt=0.01, chunks_cfg=mg.ChunksCfg(*chunks) if chunks else None))


@pytest.mark.parametrize("wall", ["rigid", "periodic"])
def test_chunked_equals_all_pairs_for_finite_range(mg, orc, wall):
    """check_chunks (test/tests_rings/tests_general.jl:16-29): with a finite
    interaction range the chunk stencil sees every interacting pair."""
    w = mg.RigidWalls() if wall == "rigid" else mg.PeriodicWalls()
    s = _harm_system(mg, 300, w, 3)
    o = orc.from_system(s)
    fs = o.forces(orc.SEQUENTIAL)
    fa = o.forces(orc.ALL_PAIRS)
    assert np.max(np.abs(fs - fa)) < 1e-12
    o2 = orc.from_system(s)
    o.step(300, orc.SEQUENTIAL)
    o2.step(300, orc.ALL_PAIRS)
    d2 = np.sum((o.state()[0] - o2.state()[0]) ** 2)
    assert d2 < 1e-4


def test_threaded_equals_sequential(mg, orc):
    """check_threaded (test/tests_rings/tests_general.jl:32-45)."""
    s = _harm_system(mg, 400, mg.PeriodicWalls(), 5)
    o1 = orc.from_system(s, nthreads=1)
    o4 = orc.from_system(s, nthreads=4)
    assert np.max(np.abs(o1.forces(orc.SEQUENTIAL) - o4.forces(orc.THREADED))) < 1e-12
    o1.step(200, orc.SEQUENTIAL)
    o4.step(200, orc.THREADED)
    assert np.sum((o1.state()[0] - o4.state()[0]) ** 2) < 1e-4


def test_newton_third_law_and_momentum(mg, orc):
    s = _harm_system(mg, 500, mg.PeriodicWalls(), 7)
    o = orc.from_system(s)
    f = o.forces()
    assert np.abs(f.sum(axis=0)).max() < 1e-10
    p0 = o.state()[1].sum(axis=0)
    o.step(100)
    assert np.abs(o.state()[1].sum(axis=0) - p0).max() < 1e-9


def test_verlet_energy_conservation_lj(mg, orc):
    lj = mg.LenJonesCfg(1.0, 1.0)
    pos, geom = mg.rectangular_grid(16, 16, 0.4, mg.particle_radius(lj))
    vel = mg.fixed_speed_vel(256, 0.2, np.random.default_rng(1))
    s = mg.System(mg.SecondLawState(pos, vel), mg.SpaceCfg(mg.PeriodicWalls(), geom), lj,
                  mg.IntCfg(dt=1e-3, chunks_cfg=mg.ChunksCfg(8, 8)))
    o = orc.from_system(s)
    ke, pe = o.energies()
    e0 = ke + pe
    o.step(500)
    ke, pe = o.energies()
    assert abs(ke + pe - e0) / abs(e0) < 1e-3


def test_rigid_walls_reflect(mg, orc):
    geom = mg.RectangleCfg(10.0, 10.0)
    dyn = mg.HarmTruncCfg(1.0, 0.0, 1.0, 1.0)
    s = mg.System(mg.SecondLawState([[0.45, 5.0], [5.0, 9.9]], [[-1.0, 0.5], [0.2, 1.0]]),
                  mg.SpaceCfg(mg.RigidWalls(), geom), dyn, mg.IntCfg(dt=0.01))
    o = orc.from_system(s)
    o.step(1)
    _, v, _ = o.state()
    assert v[0, 0] == 1.0 and v[0, 1] == 0.5     # left wall: x flipped
    assert v[1, 0] == 0.2 and v[1, 1] == -1.0    # top wall: y flipped


def test_periodic_wrap(mg, orc):
    geom = mg.RectangleCfg(10.0, 10.0)
    dyn = mg.HarmTruncCfg(1.0, 0.0, 1.0, 1.0)
    s = mg.System(mg.SecondLawState([[9.995, 5.0], [5.0, 0.002]], [[1.0, 0.0], [0.0, -1.0]]),
                  mg.SpaceCfg(mg.PeriodicWalls(), geom), dyn, mg.IntCfg(dt=0.01, chunks_cfg=mg.ChunksCfg(4, 4)))
    o = orc.from_system(s)
    o.step(1)
    p, _, _ = o.state()
    assert p[0, 0] == pytest.approx(0.005) and p[1, 1] == pytest.approx(9.992)


@pytest.mark.parametrize("wall", ["rigid", "periodic"])
def test_pair_distribution_equals_brute_force(mg, orc, wall):
    """The oracle's pair-distance histogram (chunk loop) against an independent
    all-pairs count in numpy with the same IEEE operations: the minimum image
    as calc_diff forms it, d = sqrt(dx*dx + dy*dy), bin floor(d / dr)."""
    w = mg.RigidWalls() if wall == "rigid" else mg.PeriodicWalls()
    s = _harm_system(mg, 300, w, 7)
    L, r_max, nb = 24.0, 2.0, 40
    o = orc.from_system(s)
    counts = o.pair_distribution(r_max, nb)
    p = s.state.pos
    i, j = np.triu_indices(len(p), 1)
    d = p[i] - p[j]
    if wall == "periodic":
        d = d - np.where(np.abs(d) > L / 2, np.copysign(L, d), 0.0)
    dist = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1])
    k = np.minimum((dist[dist < r_max] / (r_max / nb)).astype(np.int64), nb - 1)
    expect = np.bincount(k, minlength=nb).astype(np.uint64)
    assert counts.sum() > 0 and np.array_equal(counts, expect)
    o.close()
