"""Seeded synthetic workloads with the shapes of the benchmark configurations.

  lj_1024        2D LJ gas, 32x32 rectangular_grid (offset 0.4), |v| = 0.2 at
                 uniform angles, rigid box, velocity Verlet dt = 1e-3, chunks
                 17x17 (chunk side >= 2.5 sigma).
  harm_262144    2D harmonic-truncated soft disks (radius 1, k_rep = 10,
                 k_atr = 0, range 2r), N = 262,144 uniform in a periodic square
                 at area fraction 0.70, relaxed by 200 overdamped steps;
                 overdamped mobility 1, dt = 1e-2, chunks 542x542.
  lj_4194304     2D LJ, 2048x2048 grid (offset 0.4), periodic box, Maxwell
                 velocities T = 0.5, Verlet dt = 5e-4, chunks 1103x1103
                 (lj_262144: the same at 512x512, for profiling).
  lj_batch_512   512 LJ replicas, N log-uniform in [1000, 65536], density
                 0.6, rigid/periodic x rectangle/circle, Maxwell T in
                 [0.3, 1.0], dt = 1e-3, one handle.
  rings_64       64 replicas of a binary ring mixture (30 particles per
                 ring, 100..2000 rings), circular space with an inside
                 PotentialWalls container, springs k = 20, l = 1, area term
                 with 20% different target areas, bending, v0 = 1, D = 0.1,
                 HarmTrunc excluded volume k = 10, overdamped dt = 5e-3.
"""
from __future__ import annotations

import math

import numpy as np

from . import configs as cf
from .init_states import fixed_speed_vel, maxwell_vel, rectangular_grid
from .states import SecondLawState
from .system import System, OverdampedStep, newton_step

OVERDAMPED = OverdampedStep()


def lj_1024(precision="fp64", seed=1, use_graph=True):
    lj = cf.LenJonesCfg(1.0, 1.0)
    pos, geom = rectangular_grid(32, 32, 0.4, cf.particle_radius(lj))
    vel = fixed_speed_vel(1024, 0.2, np.random.default_rng(seed))
    return System(SecondLawState(pos, vel), cf.SpaceCfg(cf.RigidWalls(), geom), lj,
                  cf.IntCfg(dt=1e-3, chunks_cfg=cf.ChunksCfg(17, 17),
                            device=cf.CUDADevice(precision=precision, use_graph=use_graph))), newton_step


def harm_262144_initial(n=262144, phi=0.70, seed=2):
    """Uniform random positions (unrelaxed) and the box side."""
    L = math.sqrt(n * math.pi / phi)
    pos = np.random.default_rng(seed).random((n, 2)) * L
    return np.ascontiguousarray(pos), L


def harm_system(pos, L, precision="fp64", use_graph=True):
    n = pos.shape[0]
    dyn = cf.HarmTruncCfg(k_rep=10.0, k_atr=0.0, dist_eq=2.0, dist_max=2.0, mobility=1.0)
    nc = int(L // 2.0)
    return System(SecondLawState(pos.copy(), None), cf.SpaceCfg(cf.PeriodicWalls(), cf.RectangleCfg(L, L)),
                  dyn, cf.IntCfg(dt=1e-2, chunks_cfg=cf.ChunksCfg(nc, nc),
                                 device=cf.CUDADevice(precision=precision, use_graph=use_graph)))


def harm_262144(precision="fp64", relax_steps=200, n=262144, seed=2, use_graph=True):
    """Relaxed soft-disk packing (the relaxation runs on the GPU in FP64)."""
    pos, L = harm_262144_initial(n=n, seed=seed)
    s = harm_system(pos, L, "fp64", use_graph)
    if relax_steps:
        s.run(relax_steps, OVERDAMPED)
    relaxed = s.state.pos.copy()
    s.close()
    return harm_system(relaxed, L, precision, use_graph), OVERDAMPED


def lj_4194304(precision="fp64", seed=3, use_graph=True, side=2048):
    lj = cf.LenJonesCfg(1.0, 1.0)
    pos, geom = rectangular_grid(side, side, 0.4, cf.particle_radius(lj))
    vel = maxwell_vel(side * side, 0.5, np.random.default_rng(seed))
    nc = int(geom.length // 2.5)
    return System(SecondLawState(pos, vel), cf.SpaceCfg(cf.PeriodicWalls(), geom), lj,
                  cf.IntCfg(dt=5e-4, chunks_cfg=cf.ChunksCfg(nc, nc),
                            device=cf.CUDADevice(precision=precision, use_graph=use_graph))), newton_step


def _jittered_points_in_rect(n, L, rng, spacing):
    side = int(math.ceil(math.sqrt(n)))
    a = L / side
    g = (np.arange(side) + 0.5) * a
    pts = np.stack(np.meshgrid(g, g), axis=-1).reshape(-1, 2)
    pts = pts[rng.permutation(len(pts))[:n]]
    return pts + rng.uniform(-0.1, 0.1, pts.shape) * min(a - spacing, 0.5)


def lj_batch(num_replicas=512, precision="mixed", seed=4, n_min=1000, n_max=65536, density=0.6,
             use_graph=True, quadrants=("rigid_rect", "periodic_rect", "rigid_circle", "periodic_circle")):
    """Replicas of uneven N; quadrant k of the replica index picks wall x geometry."""
    rng = np.random.default_rng(seed)
    lj = cf.LenJonesCfg(1.0, 1.0)
    systems = []
    for r in range(num_replicas):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        T = rng.uniform(0.3, 1.0)
        q = quadrants[r % len(quadrants)]
        area = n / density
        if q.endswith("rect"):
            L = math.sqrt(area)
            pos = _jittered_points_in_rect(n, L, rng, 1.0)
            geom = cf.RectangleCfg(L, L)
            box = L
        else:
            R = math.sqrt(area / math.pi) * 1.05
            L = 2 * R
            side = int(math.ceil(math.sqrt(n * 4 / math.pi * 1.15)))
            a = L / side
            g = -R + (np.arange(side) + 0.5) * a
            pts = np.stack(np.meshgrid(g, g), axis=-1).reshape(-1, 2)
            pts = pts[np.sum(pts * pts, axis=1) < (R - 0.7) ** 2]
            pos = pts[rng.permutation(len(pts))[:n]]
            n = pos.shape[0]
            geom = cf.CircleCfg(R, (0.0, 0.0))
            box = L
        wall = cf.RigidWalls() if q.startswith("rigid") else cf.PeriodicWalls()
        nc = max(3, int(box // 2.5))
        vel = maxwell_vel(n, T, rng)
        systems.append(System(SecondLawState(pos, vel), cf.SpaceCfg(wall, geom), lj,
                              cf.IntCfg(dt=1e-3, chunks_cfg=cf.ChunksCfg(nc, nc),
                                        device=cf.CUDADevice(precision=precision, use_graph=use_graph))))
    return systems, newton_step


def rings_batch(num_replicas=64, precision="mixed", seed=5, n_per_ring=30, rings_min=100, rings_max=2000,
                use_graph=True, k_bend=1.0):
    """Binary ring mixtures in circular containers (inside PotentialWalls)."""
    from . import rings as R
    rng = np.random.default_rng(seed)
    inter = cf.HarmTruncCfg(k_rep=10.0, k_atr=0.0, dist_eq=1.0, dist_max=1.0)
    p0_eq = R.get_equilibrium_p0(n_per_ring)
    # type-2 target area 20% larger: area0 ~ p0^-2
    p0 = [p0_eq, p0_eq / math.sqrt(1.2)]
    cfg = R.RingsCfg(p0=p0, relax_time=[1.0, 1.0], vo=[1.0, 1.0], mobility=[1.0, 1.0], rot_diff=[0.1, 0.1],
                     k_area=[1.0, 1.0], k_spring=[20.0, 20.0], l_spring=[1.0, 1.0], k_bend=[k_bend, k_bend],
                     num_particles=[n_per_ring, n_per_ring],
                     interaction_finder=R.InteractionMatrix([[inter, inter], [inter, inter]]))
    ring_r = R.get_ring_radius(0.5, n_per_ring)
    systems = []
    for _ in range(num_replicas):
        nr = int(rng.integers(rings_min, rings_max + 1))
        spacing = 2 * (ring_r + 0.5) * 1.05
        side = int(math.ceil(math.sqrt(nr)))
        Lg = side * spacing
        Rc = Lg / math.sqrt(2) + spacing
        centers = (np.stack(np.meshgrid(np.arange(side), np.arange(side)), axis=-1).reshape(-1, 2)[:nr] + 0.5) \
            * spacing - Lg / 2
        theta = 2 * math.pi * np.arange(n_per_ring) / n_per_ring
        circle = np.stack([np.cos(theta), np.sin(theta)], axis=1) * ring_r
        rp = centers[:, None, :] + circle[None, :, :]
        types = rng.integers(1, 3, nr)
        state = R.RingsState(rp, rng.random(nr) * 2 * math.pi, num_particles=[n_per_ring, n_per_ring], types=types)
        wall = cf.PotentialWalls(potential=cf.HarmTruncCfg(k_rep=10.0, k_atr=0.0, dist_eq=0.5, dist_max=0.5),
                                 mode="inside")
        nc = max(3, int(2 * Rc // 1.1))
        systems.append(R.RingsSystem(state, cf.SpaceCfg(wall, cf.CircleCfg(Rc, (0.0, 0.0))), cfg,
                                     R.RingsIntCfg(dt=5e-3, p_chunks_cfg=cf.ChunksCfg(nc, nc),
                                                   device=cf.CUDADevice(precision=precision, use_graph=use_graph))))
    return systems, None


def lj_262144(precision="fp64", seed=3, use_graph=True):
    """The 4,194,304-particle LJ state at 512 x 512 (profiling-size case)."""
    return lj_4194304(precision=precision, seed=seed, use_graph=use_graph, side=512)


WORKLOADS = {
    "lj_1024": lj_1024,
    "harm_262144": harm_262144,
    "lj_262144": lj_262144,
    "lj_4194304": lj_4194304,
    "lj_batch_512": lj_batch,
    "rings_64": rings_batch,
}
