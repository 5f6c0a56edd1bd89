"""System, step functions and run loop mirroring Mavi.Systems / Integration /
RunSystem (src/systems.jl, src/integration.jl:507-548, src/run_system.jl).

A ``System`` owns its host state; the first step (or force / chunk / energy
query) creates a libmavi_cuda.so handle for it and uploads the state. Steps
run on the GPU; ``system.state`` is refreshed from the device after each
call, so host arrays stay authoritative between calls, as the reference's
serializers expect (src/serder.jl:59-63).

``SystemBatch`` advances many independent systems (replicas) with one handle:
one launch per kernel for all of them.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import abi, tuning
from .configs import CUDADevice, IntCfg, SpaceCfg, particle_radius, chunk_capacity
from .states import SecondLawState, SelfPropelledState


# ---------------------------------------------------------------------------
# step functions (src/integration.jl:507-548)
# ---------------------------------------------------------------------------
class StepFunction:
    kind: int = -1
    name = "step"

    def __call__(self, system, num_steps: int = 1):
        system.run(num_steps, self)

    def __repr__(self):
        return self.name


class _Newton(StepFunction):
    """newton_step!: two force passes per velocity-Verlet step (src/integration.jl:507-515)."""
    kind = abi.MAVI_STEP_NEWTON
    name = "newton_step!"


class _Szabo(StepFunction):
    """szabo_step! (src/integration.jl:517-525)."""
    kind = abi.MAVI_STEP_SZABO
    name = "szabo_step!"


class _RTP(StepFunction):
    """rtp_step! (src/integration.jl:527-535)."""
    kind = abi.MAVI_STEP_RTP
    name = "rtp_step!"


class _Rings(StepFunction):
    """Rings.Integration.step! (src/rings/integration.jl:522-543)."""
    kind = abi.MAVI_STEP_RINGS
    name = "rings step!"


class OverdampedStep(StepFunction):
    """Overdamped step composed from reference pieces, the way a user writes a
    custom step (README.md:331-332, examples/custom_step_function.jl:43-61):
    clean_forces! -> update_chunks! -> calc_forces! -> calc_walls_forces! ->
    x += mobility * F * dt -> walls! -> update_time!. The mobility is the
    dynamic config's ``mobility`` field."""
    kind = abi.MAVI_STEP_OVERDAMPED
    name = "overdamped_step!"


newton_step = _Newton()
szabo_step = _Szabo()
rtp_step = _RTP()
rings_step = _Rings()
overdamped_step = OverdampedStep()


def get_step_function(system) -> StepFunction:
    """get_step_function (src/integration.jl:537-548; rings :545)."""
    from .configs import RunTumbleCfg, SzaboCfg
    if getattr(system, "is_rings", False):
        return rings_step
    if isinstance(system.state, SecondLawState) and system.state.vel is None:
        return overdamped_step      # positions-only state: only the overdamped step applies
    if isinstance(system.dynamic_cfg, SzaboCfg):
        return szabo_step
    if isinstance(system.dynamic_cfg, RunTumbleCfg):
        return rtp_step
    return newton_step


@dataclass
class TimeInfo:
    num_steps: int = 0
    time: float = 0.0


def _check(lib, handle, st, what):
    if st != abi.MAVI_OK:
        msg = ""
        if handle:
            buf = C.create_string_buffer(512)
            lib.mavi_last_error(handle, buf, 512)
            msg = buf.value.decode()
        raise abi.MaviError(st, f"{what}: {lib.mavi_status_string(st).decode()} {msg}".strip())


class _Handle:
    """A libmavi_cuda.so handle over one or more systems."""

    def __init__(self, systems, step_kind: int, device: CUDADevice):
        self.lib = abi.load_library()
        self.systems = list(systems)
        self.step_kind = step_kind
        self.device = device
        n = len(self.systems)
        self.params = (abi.MaviReplicaParams * n)()
        for k, s in enumerate(self.systems):
            s.fill_params(self.params[k], step_kind)
        pos = np.ascontiguousarray(np.concatenate([s.state.pos.reshape(-1) for s in self.systems]))
        vel = pol = types = None
        if self.systems[0].state.kind == abi.MAVI_STATE_SECOND_LAW and self.systems[0].state.vel is not None:
            vel = np.ascontiguousarray(np.concatenate([s.state.vel.reshape(-1) for s in self.systems]))
        p0 = self.systems[0].state.pol_array()
        if p0 is not None:
            pol = np.ascontiguousarray(np.concatenate([s.state.pol_array() for s in self.systems]))
        if getattr(self.systems[0], "is_rings", False):
            types = np.ascontiguousarray(np.concatenate([s.state.types_array() for s in self.systems]).astype(np.int32))
        self.handle = C.c_void_p()
        opt, cache, key = tuning.tuned_options(self.systems, step_kind, device)
        st = self.lib.mavi_create(C.byref(opt), n, self.params, abi.as_dptr(pos), abi.as_dptr(vel),
                                  abi.as_dptr(pol), abi.as_iptr(types), C.byref(self.handle))
        _check(self.lib, None, st, "mavi_create")
        tuning.record(cache, key, self.stats())
        self.slot_offsets = np.cumsum([0] + [s.num_slots for s in self.systems])
        self.pol_offsets = np.cumsum([0] + [s.num_pol for s in self.systems])
        for k, s in enumerate(self.systems):   # per-replica clocks, then configuration (rings)
            ti = s.time_info
            if ti.num_steps or ti.time:
                self.check(self.lib.mavi_set_time(self.handle, k, int(ti.num_steps), float(ti.time)), "mavi_set_time")
            hook = getattr(s, "_configure_replica", None)
            if hook is not None:
                hook(self, k)

    def close(self):
        if self.handle:
            self.lib.mavi_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st, what):
        _check(self.lib, self.handle, st, what)

    def download(self):
        n2 = int(self.slot_offsets[-1])
        pos = np.zeros((n2, 2))
        s0 = self.systems[0].state
        vel = np.zeros((n2, 2)) if (s0.kind == abi.MAVI_STATE_SECOND_LAW and s0.vel is not None) else None
        pol = np.zeros(int(self.pol_offsets[-1])) if self.pol_offsets[-1] > 0 else None
        self.check(self.lib.mavi_download_state(self.handle, abi.as_dptr(pos), abi.as_dptr(vel), abi.as_dptr(pol)),
                   "mavi_download_state")
        for k, s in enumerate(self.systems):
            a, b = self.slot_offsets[k], self.slot_offsets[k + 1]
            s.state.pos[...] = pos[a:b]
            if vel is not None:
                s.state.vel[...] = vel[a:b]
            if pol is not None:
                s.state.pol_array()[...] = pol[self.pol_offsets[k]:self.pol_offsets[k + 1]]

    def download_async(self, pos, vel=None, pol=None):
        """Queue the copy of the device state into the given arrays (user
        order, the layout of mavi_create; page-locked memory for a copy that
        overlaps other work) and return; the arrays hold the state after
        synchronize()."""
        self.check(self.lib.mavi_download_state_async(self.handle, abi.as_dptr(pos), abi.as_dptr(vel),
                                                      abi.as_dptr(pol)), "mavi_download_state_async")

    def synchronize(self):
        """Wait for the handle's queued work; raises on a device error of it."""
        self.check(self.lib.mavi_synchronize(self.handle), "mavi_synchronize")

    def upload(self):
        pos = np.ascontiguousarray(np.concatenate([s.state.pos.reshape(-1) for s in self.systems]))
        vel = pol = None
        if self.systems[0].state.kind == abi.MAVI_STATE_SECOND_LAW and self.systems[0].state.vel is not None:
            vel = np.ascontiguousarray(np.concatenate([s.state.vel.reshape(-1) for s in self.systems]))
        if self.systems[0].state.pol_array() is not None:
            pol = np.ascontiguousarray(np.concatenate([s.state.pol_array() for s in self.systems]))
        self.check(self.lib.mavi_upload_state(self.handle, abi.as_dptr(pos), abi.as_dptr(vel), abi.as_dptr(pol)),
                   "mavi_upload_state")
        for k, s in enumerate(self.systems):   # and the clocks (a restored checkpoint's time_info)
            ti = s.time_info
            self.check(self.lib.mavi_set_time(self.handle, k, int(ti.num_steps), float(ti.time)), "mavi_set_time")

    def noise_count(self) -> int:
        return int(self.lib.mavi_noise_count(self.handle))

    def set_noise(self, noise):
        noise = np.ascontiguousarray(np.asarray(noise, dtype=np.float64).reshape(-1))
        self.check(self.lib.mavi_set_noise(self.handle, abi.as_dptr(noise), noise.size), "mavi_set_noise")

    def step(self, n: int):
        self.check(self.lib.mavi_step(self.handle, int(n)), "mavi_step")

    def forces(self, include_walls: bool) -> np.ndarray:
        out = np.zeros((int(self.slot_offsets[-1]), 2))
        self.check(self.lib.mavi_calc_forces(self.handle, 1 if include_walls else 0, abi.as_dptr(out)),
                   "mavi_calc_forces")
        return out

    def chunks(self, replica: int):
        rows, cols, cap = C.c_int32(), C.c_int32(), C.c_int32()
        self.check(self.lib.mavi_chunk_geometry(self.handle, replica, C.byref(rows), C.byref(cols), C.byref(cap)),
                   "mavi_chunk_geometry")
        r, c, k = rows.value, cols.value, cap.value
        counts = np.zeros(r * c, dtype=np.int32)
        members = np.zeros(r * c * k, dtype=np.int32)
        self.check(self.lib.mavi_get_chunks(self.handle, replica, abi.as_iptr(counts), abi.as_iptr(members)),
                   "mavi_get_chunks")
        # Julia layout: num_particles_in_chunk[rows, cols], chunk_particles[cap, rows, cols]
        return counts.reshape(c, r).T.copy(), members.reshape(c, r, k).transpose(2, 1, 0).copy()

    def energies(self, pe_mode: int):
        n = len(self.systems)
        ke = np.zeros(n)
        pe = np.zeros(n)
        self.check(self.lib.mavi_energies(self.handle, pe_mode, abi.as_dptr(ke), abi.as_dptr(pe)), "mavi_energies")
        return ke, pe

    def pass_modes(self) -> list:
        """The pass modes the autotuner chooses among for this handle: the three
        per-particle gathers; the Newton's-third-law tiles for mixed
        Lennard-Jones / WCA with chunks in every replica; 2 or 4 lanes per
        particle for the mixed harmonic-truncated and Szabo passes; the split
        gather (far pairs in FP32) for mixed Lennard-Jones."""
        modes = ["staged", "global", "columns"]
        kind = self.systems[0].dynamic_cfg.__class__.__name__
        if self.device.precision == "mixed":
            if kind in ("LenJonesCfg", "RunTumbleCfg") and all(
                    getattr(s.int_cfg, "chunks_cfg", None) is not None for s in self.systems):
                modes += ["tiles", "tiles_queue"]
            if kind in ("HarmTruncCfg", "SzaboCfg"):
                modes += ["lanes2", "lanes4"]
            if kind == "LenJonesCfg":
                modes += ["split"]
        return modes

    def stats(self) -> abi.MaviStats:
        st = abi.MaviStats()
        self.check(self.lib.mavi_get_stats(self.handle, C.byref(st)), "mavi_get_stats")
        return st

    def energy_series(self, num_samples: int, steps_between: int, pe_mode: int):
        n = len(self.systems)
        ke = np.zeros((int(num_samples), n))
        pe = np.zeros((int(num_samples), n))
        self.check(self.lib.mavi_energy_series(self.handle, int(num_samples), int(steps_between), pe_mode,
                                               abi.as_dptr(ke), abi.as_dptr(pe)), "mavi_energy_series")
        return ke, pe

    def pair_distribution(self, replica: int, r_max: float, num_bins: int) -> np.ndarray:
        out = np.zeros(int(num_bins), dtype=np.uint64)
        self.check(self.lib.mavi_pair_distribution(self.handle, int(replica), float(r_max), int(num_bins),
                                                   out.ctypes.data_as(C.POINTER(C.c_uint64))),
                   "mavi_pair_distribution")
        return out


class System:
    """A particle system (src/systems.jl:45-114) whose step loop runs on the GPU."""

    is_rings = False

    def __init__(self, state, space_cfg: SpaceCfg, dynamic_cfg, int_cfg: IntCfg, time_info: TimeInfo | None = None):
        if not isinstance(int_cfg.device, CUDADevice):
            raise TypeError("int_cfg.device must be a CUDADevice: this package runs the step loop on the GPU only")
        self.state = state
        self.space_cfg = space_cfg
        self.dynamic_cfg = dynamic_cfg
        self.int_cfg = int_cfg
        self.time_info = time_info or TimeInfo()
        self._handle: _Handle | None = None
        self._batch = None

    # ---- parameters ------------------------------------------------------
    @property
    def num_slots(self) -> int:
        return self.state.num_particles

    @property
    def num_pol(self) -> int:
        p = self.state.pol_array()
        return 0 if p is None else p.shape[0]

    def fill_params(self, p: abi.MaviReplicaParams, step_kind: int):
        C.memset(C.addressof(p), 0, C.sizeof(p))
        p.num_particles = self.num_slots
        p.state_kind = self.state.kind
        p.step_kind = step_kind
        p.dt = float(self.int_cfg.dt)
        cc = self.int_cfg.chunks_cfg
        if cc is not None:
            p.chunk_cols, p.chunk_rows = int(cc.num_cols), int(cc.num_rows)
        self.space_cfg.fill(p)
        self.dynamic_cfg.fill(p.dyn)

    def chunk_capacity(self) -> int:
        bb = self.space_cfg.bounding_box()
        cc = self.int_cfg.chunks_cfg
        return chunk_capacity(bb.length / cc.num_cols, bb.height / cc.num_rows, particle_radius(self.dynamic_cfg))

    # ---- handle ----------------------------------------------------------
    def _ensure(self, step_kind: int | None = None) -> _Handle:
        if self._batch is not None:
            raise RuntimeError("this system is driven by a SystemBatch")
        if step_kind is None:
            step_kind = self._handle.step_kind if self._handle else get_step_function(self).kind
        if self._handle is None or self._handle.step_kind != step_kind:
            if self._handle is not None:
                self._handle.close()
            self._handle = _Handle([self], step_kind, self.int_cfg.device)
        return self._handle

    def close(self):
        if self._handle is not None:
            self._handle.close()
            self._handle = None

    # ---- the reference's operations ----------------------------------------
    def run(self, num_steps: int, step_func: StepFunction | None = None, noise=None):
        step_func = step_func or get_step_function(self)
        h = self._ensure(step_func.kind)
        if noise is not None:
            h.set_noise(noise)
        h.step(num_steps)
        h.download()
        for _ in range(int(num_steps)):
            self.time_info.time += self.int_cfg.dt
            self.time_info.num_steps += 1

    def upload(self):
        """Push host-side edits of ``state`` to the device."""
        if self._handle is not None:
            self._handle.upload()

    def calc_forces(self, include_walls: bool = False) -> np.ndarray:
        """clean_forces! + update_chunks! + calc_forces! (+ calc_walls_forces!)."""
        return self._ensure().forces(include_walls)

    def chunks(self):
        """(num_particles_in_chunk[rows, cols], chunk_particles[cap, rows, cols]),
        0-based ids, -1 past each chunk's count (src/chunks.jl:23-24)."""
        return self._ensure().chunks(0)

    def energies(self, pe_mode=abi.MAVI_PE_STENCIL):
        ke, pe = self._ensure().energies(pe_mode)
        return float(ke[0]), float(pe[0])

    def stats(self) -> abi.MaviStats:
        return self._ensure().stats()

    def energy_series(self, num_samples: int, steps_between: int, step_func: StepFunction | None = None,
                      pe_mode=abi.MAVI_PE_STENCIL):
        """Advance num_samples * steps_between steps and return the kinetic and
        potential energy after every steps_between steps (arrays of
        num_samples), recorded on the device without a host round trip per
        sample (mavi_energy_series); the state is downloaded once at the end."""
        h = self._ensure(step_func.kind if step_func is not None else None)
        ke, pe = h.energy_series(num_samples, steps_between, pe_mode)
        h.download()
        for _ in range(int(num_samples) * int(steps_between)):
            self.time_info.time += self.int_cfg.dt
            self.time_info.num_steps += 1
        return ke[:, 0], pe[:, 0]

    def pair_distribution(self, r_max: float, num_bins: int) -> np.ndarray:
        """Pair-distance histogram (num_bins uint64 counts of unordered pairs per
        bin of width r_max / num_bins) of the current state; pair_correlation()
        turns it into g(r)."""
        return self._ensure().pair_distribution(0, r_max, num_bins)

    @property
    def handle(self) -> _Handle:
        return self._ensure()


class SystemBatch:
    """Many independent systems advanced by one handle (one launch per kernel
    for all replicas). All systems must share state, dynamics and step kinds;
    sizes, boxes, walls and geometries may differ."""

    def __init__(self, systems, step_func: StepFunction | None = None, device: CUDADevice | None = None):
        self.systems = list(systems)
        step_func = step_func or get_step_function(self.systems[0])
        device = device or self.systems[0].int_cfg.device
        self._handle = _Handle(self.systems, step_func.kind, device)
        for s in self.systems:
            s._batch = self

    @property
    def handle(self) -> _Handle:
        return self._handle

    def run(self, num_steps: int, noise=None, download: bool = True):
        if noise is not None:
            self._handle.set_noise(noise)
        self._handle.step(num_steps)
        if download:
            self._handle.download()
        for s in self.systems:
            for _ in range(int(num_steps)):
                s.time_info.time += s.int_cfg.dt
                s.time_info.num_steps += 1

    def calc_forces(self, include_walls: bool = False):
        f = self._handle.forces(include_walls)
        offs = self._handle.slot_offsets
        return [f[offs[k]:offs[k + 1]] for k in range(len(self.systems))]

    def energies(self, pe_mode=abi.MAVI_PE_STENCIL):
        return self._handle.energies(pe_mode)

    def energy_series(self, num_samples: int, steps_between: int, pe_mode=abi.MAVI_PE_STENCIL, download=True):
        """Per-replica (num_samples, num_replicas) kinetic and potential energy
        after every steps_between steps (mavi_energy_series)."""
        ke, pe = self._handle.energy_series(num_samples, steps_between, pe_mode)
        if download:
            self._handle.download()
        for s in self.systems:
            for _ in range(int(num_samples) * int(steps_between)):
                s.time_info.time += s.int_cfg.dt
                s.time_info.num_steps += 1
        return ke, pe

    def pair_distribution(self, r_max: float, num_bins: int, replica: int = -1) -> np.ndarray:
        """Pair-distance histogram of one replica, or of all replicas summed (-1)."""
        return self._handle.pair_distribution(replica, r_max, num_bins)

    def close(self):
        self._handle.close()
        for s in self.systems:
            s._batch = None


def run_system(system, tf=None, num_steps=None, step_func: StepFunction | None = None):
    """run_system(system; tf, num_steps, step_func) (src/run_system.jl:7-23).

    With ``tf`` the number of steps is found by accumulating dt exactly as the
    reference's ``while time < tf`` loop does, then all steps run in one call."""
    if tf is not None:
        t = system.time_info.time
        n = 0
        while t < tf:
            t += system.int_cfg.dt
            n += 1
        num_steps = n
    system.run(int(num_steps), step_func)


def kinetic_energy(obj) -> float:
    """kinetic_energy (src/quantities.jl:12-18): host state or a System (GPU)."""
    if isinstance(obj, System):
        return obj.energies()[0]
    v = obj.vel
    return 0.0 if v is None else float(np.sum(v * v) / 2)


def potential_energy(system: System, pe_mode=abi.MAVI_PE_ALL_PAIRS) -> float:
    """potential_energy (src/quantities.jl:21-66). The reference sums all pairs
    (pe_mode=MAVI_PE_ALL_PAIRS); MAVI_PE_STENCIL sums the chunk-stencil pairs
    the forces use."""
    return system.energies(pe_mode)[1]


def pair_correlation(counts, r_max: float, num_particles: int, area: float):
    """g(r) from pair-distance counts: the counts of each bin over the number
    of pairs an ideal gas at the same density would place in that annulus,
    (N / 2) (N / area) pi (r_hi^2 - r_lo^2). Returns (bin centres, g)."""
    counts = np.asarray(counts, dtype=np.float64)
    edges = np.linspace(0.0, float(r_max), counts.size + 1)
    shell = np.pi * (edges[1:] ** 2 - edges[:-1] ** 2)
    ideal = 0.5 * num_particles * (num_particles / float(area)) * shell
    return 0.5 * (edges[1:] + edges[:-1]), counts / ideal

