"""ctypes mirror of include/mavi_cuda.h and the loader of libmavi_cuda.so.

The structs here must match the C header byte for byte; tests compare their
sizes with the ones the C compiler reports. The library is loaded from the
package's own ``lib/`` directory (built in-tree by ``build.py``). There is no
CPU fallback: when the library or a GPU is missing, calls fail loudly.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib

# ---- status codes (include/mavi_cuda.h) -----------------------------------
MAVI_OK = 0
MAVI_ERR_INVALID_ARG = 1
MAVI_ERR_CUDA = 2
MAVI_ERR_OUT_OF_GRID = 3
MAVI_ERR_CHUNK_OVERFLOW = 4
MAVI_ERR_NONFINITE = 5
MAVI_ERR_OUTSIDE_SPACE = 6
MAVI_ERR_UNSUPPORTED = 7
MAVI_ERR_NO_DEVICE = 8
MAVI_ERR_NOISE_MISSING = 9
MAVI_ERR_NEIGHBOR_OVERFLOW = 10
MAVI_ERR_OFFSET_RANGE = 11
MAVI_ERR_FORCE_RANGE = 12
MAVI_MAX_NEIGHBORS = 15

MAVI_STATE_SECOND_LAW = 0
MAVI_STATE_SELF_PROPELLED = 1
MAVI_STATE_RINGS = 2

MAVI_DYN_HARM_TRUNC = 0
MAVI_DYN_LEN_JONES = 1
MAVI_DYN_SZABO = 2
MAVI_DYN_RUN_TUMBLE = 3
MAVI_DYN_RINGS = 4

MAVI_STEP_NEWTON = 0
MAVI_STEP_SZABO = 1
MAVI_STEP_RTP = 2
MAVI_STEP_RINGS = 3
MAVI_STEP_OVERDAMPED = 4

MAVI_GEOM_RECTANGLE = 0
MAVI_GEOM_CIRCLE = 1
MAVI_GEOM_LINES = 2

MAVI_WALL_RIGID = 0
MAVI_WALL_PERIODIC = 1
MAVI_WALL_SLIPPERY = 2
MAVI_WALL_POTENTIAL = 3

MAVI_POTMODE_OUTSIDE = 0
MAVI_POTMODE_INSIDE = 1
MAVI_POTMODE_REPULSION = 2

MAVI_PREC_FP64 = 0
MAVI_PREC_MIXED = 1

MAVI_NOISE_DEVICE = 0
MAVI_NOISE_INJECTED = 1

MAVI_PE_STENCIL = 0
MAVI_PE_ALL_PAIRS = 1

MAVI_MAX_SPACES = 4
MAVI_MAX_LINES = 16
MAVI_MAX_TYPES = 4

MAVI_SRC_SOURCE = 0
MAVI_SRC_SINK = 1
MAVI_SPAWN_POL_FIXED = 0
MAVI_SPAWN_POL_RANDOM = 1
MAVI_MAX_SOURCE_ENTRIES = 8
MAVI_MAX_SPAWN_BOXES = 64

MAVI_KERNEL_BIN_COUNT = 0
MAVI_KERNEL_BIN_SCAN = 1
MAVI_KERNEL_BIN_SCATTER = 2
MAVI_KERNEL_BIN_SORT = 3
MAVI_KERNEL_FORCE = 4
MAVI_KERNEL_UPDATE = 5
MAVI_KERNEL_OTHER = 6
MAVI_KERNEL_NAMES = ("bin_count", "bin_scan", "bin_scatter", "bin_sort", "force", "update", "other")
MAVI_NUM_KERNEL_KINDS = 7

T = MAVI_MAX_TYPES


class MaviSpace(C.Structure):
    _fields_ = [
        ("wall", C.c_int32), ("geometry", C.c_int32),
        ("length", C.c_double), ("height", C.c_double), ("bl_x", C.c_double), ("bl_y", C.c_double),
        ("radius", C.c_double), ("cx", C.c_double), ("cy", C.c_double),
        ("num_lines", C.c_int32), ("has_bbox", C.c_int32),
        ("lines", (C.c_double * 4) * MAVI_MAX_LINES),
        ("bbox_length", C.c_double), ("bbox_height", C.c_double),
        ("bbox_bl_x", C.c_double), ("bbox_bl_y", C.c_double),
        ("pot_kind", C.c_int32), ("pot_mode", C.c_int32),
        ("pot_params", C.c_double * 4),
    ]


class MaviRingsCfg(C.Structure):
    _fields_ = [
        ("num_types", C.c_int32), ("num_rings", C.c_int32), ("nmax", C.c_int32), ("_pad0", C.c_int32),
        ("num_particles", C.c_int32 * T),
        ("p0", C.c_double * T), ("relax_time", C.c_double * T), ("vo", C.c_double * T),
        ("mobility", C.c_double * T), ("rot_diff", C.c_double * T), ("k_area", C.c_double * T),
        ("k_spring", C.c_double * T), ("l_spring", C.c_double * T), ("k_bend", C.c_double * T),
        ("inter_k_rep", (C.c_double * T) * T), ("inter_k_atr", (C.c_double * T) * T),
        ("inter_dist_eq", (C.c_double * T) * T), ("inter_dist_max", (C.c_double * T) * T),
    ]


class MaviDynamicCfg(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("_pad0", C.c_int32),
        ("k_rep", C.c_double), ("k_atr", C.c_double), ("dist_eq", C.c_double), ("dist_max", C.c_double),
        ("sigma", C.c_double), ("epsilon", C.c_double),
        ("vo", C.c_double), ("mobility", C.c_double), ("relax_time", C.c_double), ("k_adh", C.c_double),
        ("r_eq", C.c_double), ("r_max", C.c_double), ("rot_diff", C.c_double),
        ("tumble_rate", C.c_double),
    ]


class MaviReplicaParams(C.Structure):
    _fields_ = [
        ("num_particles", C.c_int64),
        ("state_kind", C.c_int32), ("step_kind", C.c_int32), ("num_spaces", C.c_int32),
        ("chunk_cols", C.c_int32), ("chunk_rows", C.c_int32), ("_pad0", C.c_int32),
        ("dt", C.c_double),
        ("spaces", MaviSpace * MAVI_MAX_SPACES),
        ("dyn", MaviDynamicCfg),
        ("rings", MaviRingsCfg),
    ]


class MaviOptions(C.Structure):
    _fields_ = [
        ("precision", C.c_int32), ("noise_mode", C.c_int32), ("seed", C.c_uint64),
        ("device", C.c_int32), ("use_graph", C.c_int32), ("block_size", C.c_int32), ("gather_mode", C.c_int32),
    ]


class MaviStats(C.Structure):
    _fields_ = [
        ("candidate_pairs", C.c_int64), ("total_particles", C.c_int64), ("total_chunks", C.c_int64),
        ("max_chunk_count", C.c_int32), ("gather_mode", C.c_int32),
    ]


class MaviProfile(C.Structure):
    _fields_ = [
        ("ms", C.c_double * MAVI_NUM_KERNEL_KINDS),
        ("launches", C.c_int64 * MAVI_NUM_KERNEL_KINDS),
        ("steps", C.c_int64),
        ("step_ms", C.c_double),
        ("last_step_ms", C.c_double),
    ]


class MaviSourceEntry(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("num_boxes", C.c_int32), ("pol_mode", C.c_int32), ("geometry", C.c_int32),
        ("pol", C.c_double), ("pad", C.c_double),
        ("length", C.c_double), ("height", C.c_double), ("bl_x", C.c_double), ("bl_y", C.c_double),
        ("radius", C.c_double), ("cx", C.c_double), ("cy", C.c_double),
    ]


class MaviSpawnBox(C.Structure):
    _fields_ = [
        ("bl_x", C.c_double), ("bl_y", C.c_double), ("length", C.c_double), ("height", C.c_double),
        ("num_chunks", C.c_int32), ("_pad0", C.c_int32),
    ]


class MaviInvasion(C.Structure):
    _fields_ = [("invasor", C.c_int32), ("invaded", C.c_int32), ("p_id", C.c_int32), ("_pad0", C.c_int32)]


STRUCTS = {
    "MaviSpace": MaviSpace, "MaviRingsCfg": MaviRingsCfg, "MaviDynamicCfg": MaviDynamicCfg,
    "MaviReplicaParams": MaviReplicaParams, "MaviOptions": MaviOptions, "MaviStats": MaviStats,
    "MaviProfile": MaviProfile, "MaviSourceEntry": MaviSourceEntry, "MaviSpawnBox": MaviSpawnBox,
    "MaviInvasion": MaviInvasion,
}

# Exported entry points and their signatures (restype, argtypes).
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_vp = C.c_void_p
SIGNATURES = {
    "mavi_abi_version": (C.c_int, []),
    "mavi_status_string": (C.c_char_p, [C.c_int]),
    "mavi_create": (C.c_int, [C.POINTER(MaviOptions), C.c_int32, C.POINTER(MaviReplicaParams),
                              _dp, _dp, _dp, _ip, C.POINTER(_vp)]),
    "mavi_destroy": (C.c_int, [_vp]),
    "mavi_step": (C.c_int, [_vp, C.c_int64]),
    "mavi_update_chunks": (C.c_int, [_vp]),
    "mavi_chunk_geometry": (C.c_int, [_vp, C.c_int32, _ip, _ip, _ip]),
    "mavi_get_chunks": (C.c_int, [_vp, C.c_int32, _ip, _ip]),
    "mavi_calc_forces": (C.c_int, [_vp, C.c_int32, _dp]),
    "mavi_upload_state": (C.c_int, [_vp, _dp, _dp, _dp]),
    "mavi_download_state": (C.c_int, [_vp, _dp, _dp, _dp]),
    "mavi_download_state_async": (C.c_int, [_vp, _dp, _dp, _dp]),
    "mavi_synchronize": (C.c_int, [_vp]),
    "mavi_noise_count": (C.c_int64, [_vp]),
    "mavi_set_noise": (C.c_int, [_vp, _dp, C.c_int64]),
    "mavi_set_seed": (C.c_int, [_vp, C.c_uint64]),
    "mavi_energies": (C.c_int, [_vp, C.c_int32, _dp, _dp]),
    "mavi_energy_series": (C.c_int, [_vp, C.c_int64, C.c_int64, C.c_int32, _dp, _dp]),
    "mavi_pair_distribution": (C.c_int, [_vp, C.c_int32, C.c_double, C.c_int32, C.POINTER(C.c_uint64)]),
    "mavi_get_time": (C.c_int, [_vp, C.POINTER(C.c_int64), _dp]),
    "mavi_set_time": (C.c_int, [_vp, C.c_int32, C.c_int64, C.c_double]),
    "mavi_get_stats": (C.c_int, [_vp, C.POINTER(MaviStats)]),
    "mavi_profile_enable": (C.c_int, [_vp, C.c_int32]),
    "mavi_profile_read": (C.c_int, [_vp, C.POINTER(MaviProfile)]),
    "mavi_last_error": (C.c_int, [_vp, C.c_char_p, C.c_int32]),
    "mavi_fma_peak": (C.c_int, [C.c_int32, C.c_int32, _dp]),
    "mavi_rings_neighbors_config": (C.c_int, [_vp, C.c_int32, C.c_int32, C.c_int32, C.c_double]),
    "mavi_rings_neighbors": (C.c_int, [_vp, C.c_int32, _ip, _ip]),
    "mavi_rings_sources": (C.c_int, [_vp, C.c_int32, _ip, C.c_int32, C.POINTER(MaviSourceEntry),
                                     C.POINTER(MaviSpawnBox), _dp, _ip]),
    "mavi_rings_active": (C.c_int, [_vp, C.c_int32, _ip, _ip, _ip]),
    "mavi_rings_areas": (C.c_int, [_vp, C.c_int32, _dp]),
    "mavi_rings_invasions_config": (C.c_int, [_vp, C.c_int32, C.c_int32, C.c_int64, C.c_int32, C.c_int32]),
    "mavi_rings_invasions": (C.c_int, [_vp, C.c_int32, C.POINTER(MaviInvasion), C.c_int64,
                                       C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "mavi_chunk_lists_noalloc": (C.c_int, [C.POINTER(MaviReplicaParams), _vp, C.c_int64, _vp, _vp, _vp,
                                           C.c_char_p, C.c_int32]),
}

PACKAGE_DIR = pathlib.Path(__file__).resolve().parent
LIB_DIR = PACKAGE_DIR / "lib"
LIB_PATH = LIB_DIR / "libmavi_cuda.so"

_lib = None


class MaviError(RuntimeError):
    """A non-zero status returned by libmavi_cuda.so."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


def load_library(path: os.PathLike | str | None = None) -> C.CDLL:
    """Load libmavi_cuda.so (built in-tree); raise if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = pathlib.Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"libmavi_cuda.so not found at {p}; build it first "
            "(python -c 'import __graft_entry__ as g; g.build()'). There is no CPU fallback.")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def as_dptr(a):
    """Pointer to a C-contiguous float64 numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def as_iptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_ip)
