"""Shared builders for the parity tests: small seeded systems of every kind
the step loop supports."""
import math

import numpy as np


def lj_grid(mg, nx, ny, wall="rigid", chunks=None, precision="fp64", speed=0.2, seed=1, dt=1e-3,
            use_graph=True, offset=0.4):
    lj = mg.LenJonesCfg(1.0, 1.0)
    pos, geom = mg.rectangular_grid(nx, ny, offset, mg.particle_radius(lj))
    vel = mg.fixed_speed_vel(nx * ny, speed, np.random.default_rng(seed))
    w = mg.RigidWalls() if wall == "rigid" else mg.PeriodicWalls()
    if chunks is None:
        n = max(3, int(geom.length // 2.5))
        chunks = (n, n)
    return mg.System(mg.SecondLawState(pos, vel), mg.SpaceCfg(w, geom), lj,
                     mg.IntCfg(dt=dt, chunks_cfg=mg.ChunksCfg(*chunks) if chunks else None,
                               device=mg.CUDADevice(precision=precision, use_graph=use_graph)))


def soft_disks(mg, n, phi=0.7, precision="fp64", seed=2, dt=1e-2, wall="periodic", state="second_law"):
    L = math.sqrt(n * math.pi / phi)
    rng = np.random.default_rng(seed)
    pos = rng.random((n, 2)) * L
    dyn = mg.HarmTruncCfg(k_rep=10.0, k_atr=0.0, dist_eq=2.0, dist_max=2.0, mobility=1.0)
    geom = mg.RectangleCfg(L, L)
    ncell = int(L // 2.0)
    w = mg.PeriodicWalls() if wall == "periodic" else mg.RigidWalls()
    if state == "second_law":
        st = mg.SecondLawState(pos, np.zeros((n, 2)))
    else:
        st = mg.SelfPropelledState(pos, rng.random(n) * 2 * math.pi)
    return mg.System(st, mg.SpaceCfg(w, geom), dyn,
                     mg.IntCfg(dt=dt, chunks_cfg=mg.ChunksCfg(ncell, ncell),
                               device=mg.CUDADevice(precision=precision)))


def lj_circle(mg, n=300, precision="fp64", seed=3, wall="rigid"):
    lj = mg.LenJonesCfg(1.0, 1.0)
    R = math.sqrt(n / (0.5 * math.pi))
    rng = np.random.default_rng(seed)
    # jittered grid inside the circle
    a = 1.15
    xs = np.arange(-R + a, R - a, a)
    pts = np.array([(x, y) for x in xs for y in xs if x * x + y * y < (R - 1.0) ** 2])[:n]
    pts = pts + rng.uniform(-0.05, 0.05, pts.shape)
    vel = mg.maxwell_vel(len(pts), 0.5, rng)
    ncell = max(3, int(2 * R // 2.5))
    if wall == "rigid":
        space = mg.SpaceCfg(mg.RigidWalls(), mg.CircleCfg(R, (0.0, 0.0)))
    else:
        # SlipperyWalls on a circle is an obstacle (src/integration.jl:380-401):
        # a rigid square box with a circular obstacle in the middle (ManyWalls)
        keep = np.sum(pts * pts, axis=1) > (0.3 * R + 1.0) ** 2
        pts, vel = pts[keep], vel[keep]
        space = mg.SpaceCfg.many([(mg.RigidWalls(), mg.RectangleCfg(2 * R, 2 * R, (-R, -R))),
                                  (mg.SlipperyWalls(), mg.CircleCfg(0.3 * R, (0.0, 0.0)))])
    return mg.System(mg.SecondLawState(pts, vel), space, lj,
                     mg.IntCfg(dt=1e-3, chunks_cfg=mg.ChunksCfg(ncell, ncell), device=mg.CUDADevice(precision=precision)))


def self_propelled(mg, kind, n=400, precision="fp64", seed=4, noise="injected"):
    rng = np.random.default_rng(seed)
    L = math.sqrt(n / 0.5)
    pos = rng.random((n, 2)) * L
    pol = rng.random(n) * 2 * math.pi
    if kind == "rtp":
        # WCA particles must not overlap: start on a grid
        side = int(math.ceil(math.sqrt(n)))
        a = L / side
        g = (np.arange(side) + 0.5) * a
        pos = np.stack(np.meshgrid(g, g), axis=-1).reshape(-1, 2)[:n].copy()
    if kind == "szabo":
        dyn = mg.SzaboCfg(vo=1.0, mobility=1.0, relax_time=1.0, k_rep=10.0, k_adh=0.75, r_eq=1.0,
                          r_max=1.2, rot_diff=0.1)
        cell = 1.2
    else:
        dyn = mg.RunTumbleCfg(vo=1.0, sigma=1.0, epsilon=1.0, tumble_rate=0.5)
        cell = 1.2
    nc = int(L // cell)
    return mg.System(mg.SelfPropelledState(pos, pol), mg.SpaceCfg(mg.PeriodicWalls(), mg.RectangleCfg(L, L)), dyn,
                     mg.IntCfg(dt=1e-2, chunks_cfg=mg.ChunksCfg(nc, nc),
                               device=mg.CUDADevice(precision=precision, noise=noise, seed=7)))


def rings_normal(mg, precision="fp64", num_cols=6, num_rows=6, num_particles=10, seed=24042001, wall="periodic",
                 use_chunks=True, k_bend=0.0, noise="injected"):
    """create_system_normal (test/tests_rings/rings_utils.jl:27-99), seeded numpy RNG."""
    R = mg.rings
    inter = mg.HarmTruncCfg(k_rep=20.0, k_atr=4.0, dist_eq=1.0, dist_max=1.2)
    cfg = R.RingsCfg(p0=3.5, relax_time=1.0, vo=1.0, mobility=1.0, rot_diff=0.05, k_area=1.0, k_spring=20.0,
                     l_spring=1.0, num_particles=num_particles, interaction_finder=inter, k_bend=k_bend)
    rp, geom = R.rectangular_grid(num_cols=num_cols, num_rows=num_rows, num_particles=num_particles,
                                  p_radius=cfg.particle_radius(), pad_x=0.1, pad_y=0.1)
    rng = np.random.default_rng(seed)
    state = R.RingsState(rp, R.random_pol(num_cols * num_rows, rng))
    ncx = int(geom.length // (inter.dist_max * 1.1))
    ncy = int(geom.height // (inter.dist_max * 1.1))
    w = mg.PeriodicWalls() if wall == "periodic" else mg.SlipperyWalls()
    return R.RingsSystem(state, mg.SpaceCfg(w, geom), cfg,
                         R.RingsIntCfg(dt=0.01, p_chunks_cfg=mg.ChunksCfg(ncx, ncy) if use_chunks else None,
                                       device=mg.CUDADevice(precision=precision, noise=noise)))


def rings_types(mg, precision="fp64", seed=5, num_cols=5, num_rows=5):
    """create_system_types (test/tests_rings/rings_utils.jl:193-297), seeded numpy RNG."""
    R = mg.rings
    i1 = mg.HarmTruncCfg(k_rep=13, k_atr=0.1, dist_eq=1.0, dist_max=1.1)
    i2 = mg.HarmTruncCfg(k_rep=13, k_atr=0.1, dist_eq=0.8, dist_max=0.8 * 1.1)
    pe = i1.dist_eq / 2 + i2.dist_eq / 2
    ip = mg.HarmTruncCfg(k_rep=13, k_atr=10, dist_eq=pe, dist_max=pe * 1.2)
    finder = R.InteractionMatrix([[i1, ip], [ip, i2]])
    nps = [10, 5]
    cfg = R.RingsCfg(p0=3.5, relax_time=1.0, vo=1.0, mobility=1.0, rot_diff=0.5, k_area=1.0, k_spring=20.0,
                     l_spring=[i1.dist_eq * 0.8, i2.dist_eq * 0.8], num_particles=nps, interaction_finder=finder)
    rng = np.random.default_rng(seed)
    types = list(rng.integers(1, 3, num_cols * num_rows))
    rp, geom = R.rectangular_grid(num_cols=num_cols, num_rows=num_rows, num_particles=nps,
                                  p_radius=[i1.dist_eq / 2, i2.dist_eq / 2], types=types, pad_x=0.1, pad_y=0.1)
    state = R.RingsState(rp, R.random_pol(num_cols * num_rows, rng), num_particles=nps, types=types)
    mx = max(i1.dist_max, i2.dist_max, ip.dist_max) * 1.1
    ncx, ncy = int(geom.length // mx), int(geom.height // mx)
    return R.RingsSystem(state, mg.SpaceCfg(mg.PeriodicWalls(), geom), cfg,
                         R.RingsIntCfg(dt=0.01, p_chunks_cfg=mg.ChunksCfg(ncx, ncy),
                                       device=mg.CUDADevice(precision=precision, noise="injected")))


def rms(f):
    return float(np.sqrt(np.mean(np.sum(f * f, axis=1))))


def rel_force_err(f, ref):
    """max_i |F_i - F_i^ref| / RMS(|F^ref|)."""
    return float(np.max(np.linalg.norm(f - ref, axis=1)) / max(rms(ref), 1e-300))


def lj_lines(mg, kind="slippery", precision="fp64", seed=6, n_side=14, potential="harm"):
    """LJ gas in a rigid square box with line walls inside (ManyWalls): three
    slippery segments, or the same segments as PotentialWalls (harmonic or
    Lennard-Jones, repulsion mode)."""
    lj = mg.LenJonesCfg(1.0, 1.0)
    a = 1.3
    L = n_side * a
    rng = np.random.default_rng(seed)
    g = (np.arange(n_side) + 0.5) * a
    pts = np.stack(np.meshgrid(g, g), axis=-1).reshape(-1, 2) + rng.uniform(-0.05, 0.05, (n_side * n_side, 2))
    segs = [((0.3 * L, 0.2 * L), (0.3 * L, 0.7 * L)), ((0.55 * L, 0.5 * L), (0.85 * L, 0.8 * L)),
            ((0.5 * L, 0.15 * L), (0.8 * L, 0.15 * L))]
    # keep particles off the segments (distance > 0.6)
    def seg_dist(p, s):
        (x1, y1), (x2, y2) = s
        d = np.array([x2 - x1, y2 - y1]); t = np.clip(((p - [x1, y1]) @ d) / (d @ d), 0, 1)
        return np.linalg.norm(p - ([x1, y1] + t[:, None] * d), axis=1)
    keep = np.min(np.stack([seg_dist(pts, s) for s in segs]), axis=0) > 0.6
    pts = pts[keep]
    vel = mg.maxwell_vel(len(pts), 0.8, rng)
    lines = mg.LinesCfg(segs)
    if kind == "slippery":
        inner = (mg.SlipperyWalls(), lines)
    else:
        pot = mg.HarmTruncCfg(k_rep=20.0, k_atr=0.0, dist_eq=1.0, dist_max=1.0) if potential == "harm" \
            else mg.LenJonesCfg(0.8, 1.0)
        inner = (mg.PotentialWalls(pot, mode="repulsion"), lines)
    space = mg.SpaceCfg.many([(mg.RigidWalls(), mg.RectangleCfg(L, L, (0.0, 0.0))), inner])
    nc = max(3, int(L // 2.5))
    return mg.System(mg.SecondLawState(pts, vel), space, lj,
                     mg.IntCfg(dt=1e-3, chunks_cfg=mg.ChunksCfg(nc, nc), device=mg.CUDADevice(precision=precision)))
