"""ctypes wrapper of the oracle library — TEST INFRASTRUCTURE ONLY.

The oracle is the CPU FP64 restatement of Mavi.jl's step loop
(oracle/mavi_oracle.c). Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use it, as the checker; the product (libmavi_cuda.so and the
mavi_gb300 package) never imports or calls it.

It consumes the same MaviReplicaParams struct as the CUDA library, so one
parameter block drives both sides of every parity test.
"""
from __future__ import annotations

import ctypes as C
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent

SEQUENTIAL = 0
THREADED = 1
ALL_PAIRS = 2

_lib = None


def _load_lib():
    global _lib
    if _lib is not None:
        return _lib
    import importlib.util
    spec = importlib.util.spec_from_file_location("_oracle_build", HERE / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    path = mod.build()
    lib = C.CDLL(str(path))
    from mavi_gb300 import abi
    dp, ip, lp = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int64)
    vp = C.c_void_p
    sig = {
        "oracle_create": (vp, [C.POINTER(abi.MaviReplicaParams), dp, dp, dp, ip, C.c_int32, ip]),
        "oracle_destroy": (None, [vp]),
        "oracle_set_threads": (C.c_int32, [vp, C.c_int32]),
        "oracle_update_chunks": (C.c_int32, [vp]),
        "oracle_chunk_geometry": (C.c_int32, [vp, ip, ip, ip]),
        "oracle_get_chunks": (C.c_int32, [vp, ip, ip]),
        "oracle_get_neighbors": (C.c_int32, [vp, ip, ip]),
        "oracle_calc_forces": (C.c_int32, [vp, C.c_int32, C.c_int32, dp]),
        "oracle_noise_count": (C.c_int64, [vp]),
        "oracle_step": (C.c_int32, [vp, C.c_int64, C.c_int32, dp]),
        "oracle_get_state": (C.c_int32, [vp, dp, dp, dp]),
        "oracle_set_state": (C.c_int32, [vp, dp, dp, dp]),
        "oracle_energies": (C.c_int32, [vp, C.c_int32, dp, dp]),
        "oracle_get_time": (C.c_int32, [vp, lp, dp]),
        "oracle_set_time": (C.c_int32, [vp, C.c_int64, C.c_double]),
        "oracle_get_areas": (C.c_int32, [vp, dp]),
        "oracle_count_pairs": (C.c_int64, [vp]),
        "oracle_pair_distribution": (C.c_int32, [vp, C.c_double, C.c_int32, C.POINTER(C.c_uint64)]),
        "oracle_rings_neighbors": (C.c_int32, [vp, C.c_double, C.c_int32, C.c_int32, C.POINTER(C.c_int32),
                                               C.POINTER(C.c_int32)]),
        "oracle_rings_sources": (C.c_int32, [vp, ip, C.c_int32, C.POINTER(abi.MaviSourceEntry),
                                             C.POINTER(abi.MaviSpawnBox), dp, ip]),
        "oracle_rings_active": (C.c_int32, [vp, ip, ip, ip]),
        "oracle_rings_invasions_config": (C.c_int32, [vp, C.c_int32, C.c_int64, C.c_int32, C.c_int32]),
        "oracle_rings_invasions": (C.c_int32, [vp, C.POINTER(abi.MaviInvasion), C.c_int64, lp, lp]),
        "oracle_julia_div": (C.c_double, [C.c_double, C.c_double]),
        "oracle_chunk_of": (C.c_int32, [vp, C.c_double, C.c_double, lp, lp]),
        "oracle_struct_sizes": (C.c_int32, [lp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


class OracleError(RuntimeError):
    def __init__(self, status, what):
        super().__init__(f"oracle {what}: status {status}")
        self.status = status


class OracleSystem:
    """One replica (a Julia ``System``) on the CPU oracle."""

    def __init__(self, params, pos, vel=None, pol=None, types=None, nthreads: int = 1):
        self.lib = _load_lib()
        self.params = params
        self.n = int(params.num_particles)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
        pol = None if pol is None else np.ascontiguousarray(pol, dtype=np.float64).reshape(-1)
        self.types = None if types is None else np.ascontiguousarray(types, dtype=np.int32)
        st = C.c_int32()
        self.h = self.lib.oracle_create(C.byref(params), _dp(pos), _dp(vel), _dp(pol),
                                        None if self.types is None else self.types.ctypes.data_as(C.POINTER(C.c_int32)),
                                        int(nthreads), C.byref(st))
        self.status = st.value
        self.has_vel = vel is not None
        self.npol = 0 if pol is None else pol.size

    def close(self):
        if self.h:
            self.lib.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st, what):
        if st != 0:
            raise OracleError(st, what)

    def set_threads(self, n: int):
        self.lib.oracle_set_threads(self.h, int(n))

    def update_chunks(self):
        return self.lib.oracle_update_chunks(self.h)

    def chunk_geometry(self):
        r, c, k = C.c_int32(), C.c_int32(), C.c_int32()
        self.lib.oracle_chunk_geometry(self.h, C.byref(r), C.byref(c), C.byref(k))
        return r.value, c.value, k.value

    def chunks(self):
        """Reference layout: (num_in_chunk[rows, cols], chunk_particles[cap, rows, cols]), 0-based ids."""
        r, c, k = self.chunk_geometry()
        counts = np.zeros(r * c, dtype=np.int32)
        members = np.zeros(r * c * k, dtype=np.int32)
        self._ck(self.lib.oracle_get_chunks(self.h, counts.ctypes.data_as(C.POINTER(C.c_int32)),
                                            members.ctypes.data_as(C.POINTER(C.c_int32))), "get_chunks")
        return counts.reshape(c, r).T.copy(), members.reshape(c, r, k).transpose(2, 1, 0).copy()

    def neighbors(self):
        r, c, _ = self.chunk_geometry()
        cnt = np.zeros(r * c, dtype=np.int32)
        nb = np.zeros(r * c * 4, dtype=np.int32)
        self._ck(self.lib.oracle_get_neighbors(self.h, cnt.ctypes.data_as(C.POINTER(C.c_int32)),
                                               nb.ctypes.data_as(C.POINTER(C.c_int32))), "get_neighbors")
        return cnt, nb.reshape(r * c, 4)

    def forces(self, mode=SEQUENTIAL, include_walls=False):
        out = np.zeros(2 * self.n)
        self._ck(self.lib.oracle_calc_forces(self.h, mode, 1 if include_walls else 0, _dp(out)), "calc_forces")
        return out.reshape(-1, 2)

    def noise_count(self) -> int:
        return int(self.lib.oracle_noise_count(self.h))

    def step(self, nsteps: int = 1, mode=SEQUENTIAL, noise=None):
        """Advance nsteps; steps that draw random numbers (Szabo, RTP, rings)
        take them from `noise` (nsteps * noise_count() numbers, step-major)."""
        need = self.noise_count() * int(nsteps)
        if need and (noise is None or np.size(noise) < need):
            raise ValueError(f"this step consumes {self.noise_count()} noise numbers per step: pass {need}")
        noise = None if noise is None else np.ascontiguousarray(noise, dtype=np.float64).reshape(-1)
        st = self.lib.oracle_step(self.h, int(nsteps), mode, _dp(noise))
        self._ck(st, "step")

    def state(self):
        pos = np.zeros(2 * self.n)
        vel = np.zeros(2 * self.n) if self.has_vel else None
        pol = np.zeros(self.npol) if self.npol else None
        self.lib.oracle_get_state(self.h, _dp(pos), _dp(vel), _dp(pol))
        return pos.reshape(-1, 2), (None if vel is None else vel.reshape(-1, 2)), pol

    def set_state(self, pos, vel=None, pol=None):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
        pol = None if pol is None else np.ascontiguousarray(pol, dtype=np.float64).reshape(-1)
        self.lib.oracle_set_state(self.h, _dp(pos), _dp(vel), _dp(pol))

    def energies(self, pe_mode=0):
        ke, pe = C.c_double(), C.c_double()
        self._ck(self.lib.oracle_energies(self.h, pe_mode, C.byref(ke), C.byref(pe)), "energies")
        return ke.value, pe.value

    def time(self):
        n, t = C.c_int64(), C.c_double()
        self.lib.oracle_get_time(self.h, C.byref(n), C.byref(t))
        return n.value, t.value

    def areas(self, num_rings):
        a = np.zeros(num_rings)
        self._ck(self.lib.oracle_get_areas(self.h, _dp(a)), "areas")
        return a

    def rings_neighbors(self, tol=1.1, type_all=False, max_list=15, with_lists=True):
        """Particle neighbour counts (n) and lists (n x max_list, -1 padded,
        reference append order) of the rings model at the current state."""
        counts = np.zeros(self.n, dtype=np.int32)
        lists = np.full(self.n * max_list, -1, dtype=np.int32) if with_lists else None
        ip = C.POINTER(C.c_int32)
        st = self.lib.oracle_rings_neighbors(self.h, float(tol), 1 if type_all else 0, int(max_list),
                                             counts.ctypes.data_as(ip),
                                             lists.ctypes.data_as(ip) if lists is not None else None)
        self._ck(st, "rings_neighbors")
        return counts, (lists.reshape(self.n, max_list) if lists is not None else None)

    def count_pairs(self) -> int:
        return int(self.lib.oracle_count_pairs(self.h))

    def pair_distribution(self, r_max: float, nbins: int) -> np.ndarray:
        """Pair-distance histogram counts (num_bins uint64) of the current state."""
        out = np.zeros(int(nbins), dtype=np.uint64)
        self._ck(self.lib.oracle_pair_distribution(self.h, float(r_max), int(nbins),
                                                   out.ctypes.data_as(C.POINTER(C.c_uint64))), "pair_distribution")
        return out

    def rings_sources(self, mask, num_entries, entries, boxes, spawn_xy, chunk_rc):
        """Variable rings ids with sources and sinks (the arguments of
        mavi_rings_sources for this replica)."""
        ip = C.POINTER(C.c_int32)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        sp = np.ascontiguousarray(spawn_xy, dtype=np.float64)
        rc = np.ascontiguousarray(chunk_rc, dtype=np.int32)
        self._ck(self.lib.oracle_rings_sources(self.h, None if m is None else m.ctypes.data_as(ip), int(num_entries),
                                               entries, boxes, _dp(sp), rc.ctypes.data_as(ip)), "rings_sources")

    def rings_ids(self):
        """(active mask bool, uids, num_active)."""
        nr = self.params.rings.num_rings
        m = np.zeros(nr, dtype=np.int32)
        u = np.zeros(nr, dtype=np.int32)
        na = C.c_int32()
        ip = C.POINTER(C.c_int32)
        self._ck(self.lib.oracle_rings_active(self.h, m.ctypes.data_as(ip), u.ctypes.data_as(ip), C.byref(na)),
                 "rings_active")
        return m.astype(bool), u, int(na.value)

    def rings_invasions_config(self, enable, steps_to_update, num_cols=0, num_rows=0):
        """InvasionsCfg and ring chunks, as mavi_rings_invasions_config."""
        self._ck(self.lib.oracle_rings_invasions_config(self.h, 1 if enable else 0, int(steps_to_update),
                                                        int(num_cols), int(num_rows)), "rings_invasions_config")

    def rings_invasions(self):
        """(list of (invasor, invaded, p_id), last_check)."""
        from mavi_gb300 import abi
        n, last = C.c_int64(), C.c_int64()
        self._ck(self.lib.oracle_rings_invasions(self.h, None, 0, C.byref(n), C.byref(last)), "rings_invasions")
        out = (abi.MaviInvasion * max(n.value, 1))()
        self._ck(self.lib.oracle_rings_invasions(self.h, out, n.value, C.byref(n), C.byref(last)), "rings_invasions")
        return [(out[k].invasor, out[k].invaded, out[k].p_id) for k in range(n.value)], int(last.value)

    def chunk_of(self, x, y):
        r, c = C.c_int64(), C.c_int64()
        st = self.lib.oracle_chunk_of(self.h, float(x), float(y), C.byref(r), C.byref(c))
        return st, r.value, c.value


def julia_div(x: float, y: float) -> float:
    return _load_lib().oracle_julia_div(float(x), float(y))


def struct_sizes():
    out = (C.c_int64 * 16)()
    n = _load_lib().oracle_struct_sizes(out)
    names = ["MaviSpace", "MaviRingsCfg", "MaviDynamicCfg", "MaviReplicaParams", "MaviOptions", "MaviStats",
             "MaviProfile", "MaviSourceEntry", "MaviSpawnBox", "MaviInvasion"]
    return {names[k]: out[k] for k in range(n)}


def noise_for(kind: int, count: int, rng) -> np.ndarray:
    """Noise numbers of one step: RTP draws uniforms, Szabo and rings normals."""
    from mavi_gb300 import abi
    return rng.random(count) if kind == abi.MAVI_STEP_RTP else rng.standard_normal(count)


def from_system(system, nthreads: int = 1, step_kind=None) -> OracleSystem:
    """An oracle replica with the same parameters and state as a mavi_gb300 System."""
    from mavi_gb300 import abi
    from mavi_gb300.system import get_step_function
    p = abi.MaviReplicaParams()
    kind = step_kind if step_kind is not None else get_step_function(system).kind
    system.fill_params(p, kind)
    st = system.state
    vel = getattr(st, "vel", None)
    pol = st.pol_array()
    types = st.types_array() if getattr(system, "is_rings", False) else None
    o = OracleSystem(p, st.pos, vel, pol, types, nthreads=nthreads)
    ti = getattr(system, "time_info", None)
    if ti is not None and (ti.num_steps or ti.time):
        o.lib.oracle_set_time(o.h, int(ti.num_steps), float(ti.time))
    src = system.sources_abi() if hasattr(system, "sources_abi") else None
    if src is not None:
        o.rings_sources(*src)
    inv = system.invasions_abi() if hasattr(system, "invasions_abi") else None
    if inv is not None:
        o.rings_invasions_config(*inv)
    return o
