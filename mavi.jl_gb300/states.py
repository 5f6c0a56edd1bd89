"""Particle states mirroring Mavi.States (src/states.jl).

Positions and velocities are (N, 2) float64 C-contiguous arrays: the same
bytes as Julia's ``Vector{SVector{2,Float64}}`` ([x1, y1, x2, y2, ...],
src/states.jl:75-79), so they cross the C ABI without a copy.
"""
from __future__ import annotations

import numpy as np

from . import abi


def _as_xy(a) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if a.ndim == 2 and a.shape[0] == 2 and a.shape[1] != 2:
        a = np.ascontiguousarray(a.T)      # Julia-style (2, N) matrix
    if a.ndim != 2 or a.shape[1] != 2:
        raise ValueError("positions/velocities must have shape (N, 2)")
    return a


class SecondLawState:
    """Positions and velocities for Newton's second law (src/states.jl:75-101).

    ``vel=None`` gives a positions-only state, accepted by the overdamped step
    only (velocities play no part in it)."""
    kind = abi.MAVI_STATE_SECOND_LAW

    def __init__(self, pos, vel):
        self.pos = _as_xy(pos)
        self.vel = None if vel is None else _as_xy(vel)
        if self.vel is not None and self.pos.shape != self.vel.shape:
            raise ValueError("pos and vel must have the same number of particles")

    @property
    def num_particles(self) -> int:
        return self.pos.shape[0]

    def pol_array(self):
        return None


class SelfPropelledState:
    """Overdamped self-propelled state: positions and polarisation angles
    (src/states.jl:104-125)."""
    kind = abi.MAVI_STATE_SELF_PROPELLED

    def __init__(self, pos, pol_angle):
        self.pos = _as_xy(pos)
        self.pol_angle = np.ascontiguousarray(np.asarray(pol_angle, dtype=np.float64).reshape(-1))
        if self.pol_angle.shape[0] != self.pos.shape[0]:
            raise ValueError("pol_angle must have one entry per particle")
        self.vel = None

    @property
    def num_particles(self) -> int:
        return self.pos.shape[0]

    def pol_array(self):
        return self.pol_angle


def get_num_total_particles(state) -> int:
    return state.num_particles
