"""mavi_chunk_lists_noalloc: chunk lists of device-resident positions built
from the library's fixed scratch array, with no device allocation.

Compared, through the C ABI, with the handle-based entry point
(mavi_get_chunks) on two calls in a row with different positions; the file is
named so that it is collected last and runs the same alone or after the other
tests (the scratch is shared by every call on a device)."""
import ctypes as C

import numpy as np
import pytest

from helpers import lj_grid, soft_disks

pytestmark = pytest.mark.gpu


def _params(mg, system):
    p = mg.abi.MaviReplicaParams()
    system.fill_params(p, mg.get_step_function(system).kind)
    return p


def _noalloc(mg, params, pos_host, free_bytes=None):
    """Call the entry point on device copies of `pos_host`; returns the status,
    the message and the lists in the reference layout. With `free_bytes` (a
    list), the device's free memory just before and just after the call (the
    caller's buffers are all allocated before the first reading) is appended."""
    import torch
    lib = mg.load_library()
    rows, cols = params.chunk_rows, params.chunk_cols
    n = pos_host.shape[0]
    pos = torch.from_numpy(np.ascontiguousarray(pos_host)).cuda()
    start = torch.full((rows * cols + 1,), -7, dtype=torch.int32, device="cuda")
    ids = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    msg = C.create_string_buffer(256)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    if free_bytes is not None:
        free_bytes.append(torch.cuda.mem_get_info()[0])
    st = lib.mavi_chunk_lists_noalloc(C.byref(params), C.c_void_p(pos.data_ptr()), n,
                                      C.c_void_p(start.data_ptr()), C.c_void_p(ids.data_ptr()),
                                      stream, msg, 256)
    torch.cuda.synchronize()
    if free_bytes is not None:
        free_bytes.append(torch.cuda.mem_get_info()[0])
    return st, msg.value.decode(), start.cpu().numpy(), ids.cpu().numpy()[:n]


def _reference_layout(start, ids, rows, cols, cap):
    counts = np.zeros((rows, cols), dtype=np.int32)
    members = np.full((cap, rows, cols), -1, dtype=np.int32)
    for c in range(rows * cols):
        col, row = divmod(c, rows)
        b, e = start[c], start[c + 1]
        counts[row, col] = e - b
        members[:e - b, row, col] = ids[b:e]
    return counts, members


def _check_against_handle(mg, system):
    counts_ref, members_ref = system.chunks()          # mavi_get_chunks on the same state
    params = _params(mg, system)
    st, msg, start, ids = _noalloc(mg, params, system.state.pos)
    assert st == mg.abi.MAVI_OK, msg
    assert start[0] == 0 and start[-1] == system.num_slots
    assert np.array_equal(np.sort(ids), np.arange(system.num_slots))
    counts, members = _reference_layout(start, ids, params.chunk_rows, params.chunk_cols, members_ref.shape[0])
    assert np.array_equal(counts, counts_ref)
    assert np.array_equal(members, members_ref)


@pytest.mark.parametrize("wall", ["rigid", "periodic"])
def test_noalloc_matches_get_chunks_two_calls(mg, wall):
    s = lj_grid(mg, 32, 32, wall=wall, chunks=(17, 17), speed=1.0)
    mg.run_system(s, num_steps=30)
    _check_against_handle(mg, s)
    mg.run_system(s, num_steps=200)                    # different positions for the second call
    _check_against_handle(mg, s)
    s.close()


def test_noalloc_matches_get_chunks_soft_disks(mg):
    s = soft_disks(mg, 65536, precision="mixed")
    mg.run_system(s, num_steps=20, step_func=mg.overdamped_step)
    _check_against_handle(mg, s)
    mg.run_system(s, num_steps=20, step_func=mg.overdamped_step)
    _check_against_handle(mg, s)
    s.close()


def test_noalloc_rejects_sizes_beyond_its_scratch(mg):
    s = lj_grid(mg, 8, 8, wall="rigid", chunks=(3, 3))
    p = _params(mg, s)
    p.chunk_rows, p.chunk_cols = 1025, 1024           # 1,049,600 chunks > 1,048,576
    st, msg, _, _ = _noalloc(mg, p, s.state.pos)
    assert st == mg.abi.MAVI_ERR_INVALID_ARG and "1048576" in msg, msg
    p = _params(mg, s)
    p.dyn.sigma = 0.01                                # tiny particles: chunk capacity above 1024
    st, msg, _, _ = _noalloc(mg, p, s.state.pos)
    assert st == mg.abi.MAVI_ERR_INVALID_ARG and "capacity" in msg, msg
    s.close()


def test_noalloc_reports_particle_outside_grid(mg):
    s = lj_grid(mg, 8, 8, wall="rigid", chunks=(3, 3))
    p = _params(mg, s)
    pos = s.state.pos.copy()
    pos[5] = (1e6, 0.0)
    st, msg, _, _ = _noalloc(mg, p, pos)
    assert st == mg.abi.MAVI_ERR_OUT_OF_GRID, msg
    # the scratch is cleared by the next call: a clean call succeeds again
    _check_against_handle(mg, s)
    s.close()


def test_noalloc_leaves_free_device_memory_unchanged(mg):
    """After a first call on the device (which loads the library module holding
    the fixed scratch), a call changes the device's free memory by nothing: it
    allocates no device memory, and nothing it calls does."""
    s = soft_disks(mg, 65536, precision="fp64")
    p = _params(mg, s)
    st, msg, _, _ = _noalloc(mg, p, s.state.pos)              # set-up call
    assert st == mg.abi.MAVI_OK, msg
    free = []
    st, msg, start, ids = _noalloc(mg, p, s.state.pos, free_bytes=free)
    assert st == mg.abi.MAVI_OK, msg
    assert free[0] == free[1], free
    assert np.array_equal(np.sort(ids), np.arange(s.num_slots))
    s.close()


def test_noalloc_reports_chunk_overflow_then_recovers(mg):
    """More particles in one chunk than its capacity is the reference's
    BoundsError: the call returns MAVI_ERR_CHUNK_OVERFLOW; the next call, on a
    valid state, clears the shared scratch and succeeds."""
    s = lj_grid(mg, 8, 8, wall="rigid", chunks=(3, 3))
    p = _params(mg, s)
    cap = s.chunk_capacity()
    assert s.num_slots > cap
    g = s.space_cfg.geometry_cfg
    centre = np.array(g.bottom_left, dtype=float) + np.array([g.length / 2, g.height / 2])
    k = np.arange(s.num_slots)
    pos = centre + 0.01 * np.stack([k % 8, k // 8], axis=1)  # all in the middle chunk
    st, msg, _, _ = _noalloc(mg, p, pos)
    assert st == mg.abi.MAVI_ERR_CHUNK_OVERFLOW, msg
    assert "capacity" in msg, msg
    _check_against_handle(mg, s)
    _check_against_handle(mg, s)
    s.close()
