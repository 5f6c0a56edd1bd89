"""mavi_gb300 — Mavi.jl's step loop on one GB300 GPU.

A Julia-like host API (System, run_system, step functions, configs, states,
the rings model) over libmavi_cuda.so, the hand-written CUDA implementation
(sm_103a) of chunk rebuild -> pair forces -> integration -> walls. There is no
CPU fallback: operations fail loudly when the library or a GPU is missing.
"""
from . import abi
from .abi import MaviError, load_library
from .configs import (
    ChunksCfg, CircleCfg, CUDADevice, HarmTruncCfg, IntCfg, LenJonesCfg, LinesCfg, PeriodicWalls,
    PotentialWalls, RectangleCfg, RigidWalls, RunTumbleCfg, SlipperyWalls, SpaceCfg, SzaboCfg,
    chunk_capacity, has_chunks, particle_radius,
)
from .states import SecondLawState, SelfPropelledState, get_num_total_particles
from .system import (
    OverdampedStep, System, SystemBatch, TimeInfo, get_step_function, kinetic_energy, newton_step,
    overdamped_step, pair_correlation, potential_energy, rings_step, rtp_step, run_system, szabo_step,
)
from .init_states import fixed_speed_vel, maxwell_vel, random_vel, rectangular_grid
from . import rings
from . import replicas
from . import tuning
from . import experiments
from .experiments import (
    CheckpointCfg, DelayedCfg, Experiment, ExperimentCfg, ManyColsCfg, load_experiment, run_experiment,
)
from .replicas import my_replicas, shard_replicas

__all__ = [n for n in dir() if not n.startswith("_")]
