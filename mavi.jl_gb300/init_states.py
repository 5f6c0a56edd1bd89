"""Initial-state helpers mirroring Mavi.InitStates (src/init_states.jl) and
the seeded synthetic workloads used by the tests and the benchmark."""
from __future__ import annotations

import math

import numpy as np

from .configs import RectangleCfg


def rectangular_grid(num_p_x: int, num_p_y: int, offset: float, radius: float):
    """rectangular_grid (src/init_states.jl:34-57): positions with spacing
    ``offset*radius`` and the RectangleCfg that contains them. The running sums
    are accumulated exactly as the reference does (one row and one column are
    built sequentially, then tiled)."""
    step = radius * (2 + offset)
    xs = []
    cur = -radius
    for _ in range(num_p_x):
        cur = cur + step
        xs.append(cur)
    ys = []
    cy = radius * (offset + 1)
    for _ in range(num_p_y):
        ys.append(cy)
        cy += step
    x = np.tile(np.asarray(xs), num_p_y)
    y = np.repeat(np.asarray(ys), num_p_x)
    geom = RectangleCfg(
        length=num_p_x * 2 * radius + radius * offset * (num_p_x + 1),
        height=num_p_y * 2 * radius + radius * offset * (num_p_y + 1),
    )
    return np.ascontiguousarray(np.stack([x, y], axis=1)), geom


def random_vel(num_p: int, max_value: float = 1.0, rng=None):
    """random_vel (src/init_states.jl:63-70): components uniform in
    [-max_value, max_value] (seeded numpy generator instead of Julia's)."""
    rng = rng or np.random.default_rng()
    return (rng.random((num_p, 2)) * 2 - 1) * max_value


def fixed_speed_vel(num_p: int, speed: float, rng) -> np.ndarray:
    """Velocities of magnitude ``speed`` at uniform random angles."""
    th = rng.random(num_p) * 2 * math.pi
    return np.ascontiguousarray(np.stack([speed * np.cos(th), speed * np.sin(th)], axis=1))


def maxwell_vel(num_p: int, temperature: float, rng, remove_drift: bool = True) -> np.ndarray:
    """Maxwell-Boltzmann velocities (unit mass, k_B = 1)."""
    v = rng.normal(0.0, math.sqrt(temperature), size=(num_p, 2))
    if remove_drift:
        v -= v.mean(axis=0, keepdims=True)
    return np.ascontiguousarray(v)
