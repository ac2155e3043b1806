"""The photon-grid entry point that allocates nothing, checked against the allocating one.

rt_stage_photon_grid_noalloc serves callers that cannot allocate device memory: frame loops with a
no-allocation rule (cudaMalloc / cudaFree can synchronise the device), hosts whose device memory all
comes from their own allocator or pool, and processes near the memory limit.  It takes device
pointers and keeps its scratch in one fixed device array shared by every call, so two calls in a
row must each give the allocating entry point's result, bit for bit: the second call must not see
anything the first left in the shared array.  The test's own device buffers come from torch (the
test itself may allocate; the entry point under test does not).
"""
import ctypes as C

import numpy as np
import pytest

import rustracer_gb300 as rt
from rustracer_gb300 import _abi as A

pytestmark = pytest.mark.gpu


def photons(seed, n, gp):
    rng = np.random.default_rng(seed)
    ph = np.zeros(n, A.np_dtype(A.Photon))
    lo = np.array([gp.room_min_x, gp.room_min_y, gp.room_min_z], np.float32)
    span = np.array([gp.grid_x, gp.grid_y, gp.grid_z], np.float32) * np.float32(gp.cell_size)
    ph["position"] = lo + rng.random((n, 3), np.float32) * span * np.float32(1.1) - span * np.float32(0.05)
    ph["power"] = rng.random((n, 3), np.float32)
    ph["power"][rng.random(n) < 0.2, 0] = 0.0  # empty slots (power.r <= 0)
    ph["position"][10:1500] = lo + span * np.float32(0.5)  # one cell with more than 1024 photons
    return ph


def test_noalloc_grid_matches_allocating_entry_point_on_two_calls(gpu):
    torch = pytest.importorskip("torch")
    lib = A.load()
    dev = torch.device("cuda")
    stream = torch.cuda.current_stream()
    # Two calls in a row with different grids and photon counts.
    for seed, n, grid_max_dim, radius_mode in [(0, 200_000, 26, 0), (1, 150_000, 64, 1)]:
        gp, _ = rt.derive_grid((np.zeros(3), np.full(3, 555.0)), grid_max_dim, radius_mode, n)
        assert gp.num_cells <= A.NOALLOC_MAX_CELLS and n <= A.NOALLOC_MAX_SLOTS
        ph = photons(seed, n, gp)
        ref_counts, ref_meta, ref_sorted = rt.stage_photon_grid(ph, gp)

        d_ph = torch.from_numpy(ph.view(np.uint8).copy()).to(dev)
        d_counts = torch.full((gp.num_cells,), -1, dtype=torch.int32, device=dev)  # stale garbage
        d_meta = torch.full((2 * gp.num_cells,), -1, dtype=torch.int32, device=dev)
        d_sorted = torch.zeros((n * 64,), dtype=torch.uint8, device=dev)
        g = A.GridParams.from_buffer_copy(gp)
        g.photon_slots = n
        st = lib.rt_stage_photon_grid_noalloc(C.c_void_p(d_ph.data_ptr()), C.byref(g),
                                              C.c_void_p(d_counts.data_ptr()), C.c_void_p(d_meta.data_ptr()),
                                              C.c_void_p(d_sorted.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert st == A.RT_OK, lib.rt_last_error()
        stream.synchronize()
        counts = d_counts.cpu().numpy().view(np.uint32)
        meta = d_meta.cpu().numpy().view(np.uint32).reshape(-1, 2)
        assert np.array_equal(counts, ref_counts)
        assert np.array_equal(meta, ref_meta)
        binned = int(counts.sum())
        assert binned > 0
        assert np.array_equal(d_sorted.cpu().numpy()[: binned * 64], ref_sorted.view(np.uint8).ravel()[: binned * 64])

    # Once the library is loaded on the device, a call takes no device memory: free memory is the same
    # before and after a third call on the buffers above.
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    st = lib.rt_stage_photon_grid_noalloc(C.c_void_p(d_ph.data_ptr()), C.byref(g), C.c_void_p(d_counts.data_ptr()),
                                          C.c_void_p(d_meta.data_ptr()), C.c_void_p(d_sorted.data_ptr()),
                                          C.c_void_p(stream.cuda_stream))
    assert st == A.RT_OK, lib.rt_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    assert np.array_equal(d_counts.cpu().numpy().view(np.uint32), ref_counts)

    # Sizes beyond the fixed scratch are refused with a clear error, before any work is enqueued.
    g = A.GridParams.from_buffer_copy(gp)
    g.photon_slots = A.NOALLOC_MAX_SLOTS + 1
    st = lib.rt_stage_photon_grid_noalloc(C.c_void_p(d_ph.data_ptr()), C.byref(g), C.c_void_p(d_counts.data_ptr()),
                                          C.c_void_p(d_meta.data_ptr()), C.c_void_p(d_sorted.data_ptr()), None)
    assert st == A.RT_ERR_INVALID_ARGUMENT
    assert b"at most" in lib.rt_last_error()
