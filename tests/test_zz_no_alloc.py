"""gbh_sort_pairs_noalloc, the sort entry point that allocates nothing.

It serves callers that cannot call cudaMalloc (device memory owned by another
allocator or engine, or a loop that must not touch the allocator).  The test
sorts the same unsorted Morton keys and body indices that a step's compaction
produced, once through the context's sort stage (gbh_stage_sort, which sorts
in buffers the context allocated at creation) and twice in a row through the
allocation-free entry point on buffers the test owns.  Every result must be
identical: the sort is integer work, so the tolerance is zero.

The file is named to be collected last, and it needs no other test's state.
"""
import ctypes as C

import numpy as np
import pytest

from gravity_gb300 import BarnesHut, abi, ic

pytestmark = pytest.mark.gpu


def _unsorted_and_sorted(n, seed):
    bodies = ic.plummer(n, seed=seed)
    sim = BarnesHut(n, ic.exact_bounds(bodies), abi.units(G=1.0))
    sim.upload_bodies(bodies)
    sim.init()
    p = abi.step_params()
    sim.reset_values(p)
    sim.partition_dead_bodies(p)  # compaction + bounds + Morton keys
    keys = sim.read_morton()[:n].copy()
    idx = sim.read_index()[:n].copy()
    sim.radix_sort()  # the existing entry point
    return keys, idx, sim.read_morton()[:n].copy(), sim.read_index()[:n].copy()


def test_sort_pairs_noalloc_matches_stage_sort(gbh_lib):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.current_stream()
    for call, (n, seed) in enumerate([(300000, 5), (1 << 20, 6)]):
        keys, idx, want_k, want_v = _unsorted_and_sorted(n, seed)
        kin = torch.from_numpy(keys.view(np.int64)).cuda()
        vin = torch.from_numpy(idx.view(np.int32)).cuda()
        kout = torch.empty_like(kin)
        vout = torch.empty_like(vin)
        torch.cuda.synchronize()
        rc = gbh_lib.gbh_sort_pairs_noalloc(
            C.c_void_p(kin.data_ptr()), C.c_void_p(vin.data_ptr()), C.c_void_p(kout.data_ptr()),
            C.c_void_p(vout.data_ptr()), n, C.c_void_p(stream.cuda_stream))
        assert rc == abi.GBH_OK, (call, rc)
        got_k = kout.cpu().numpy().view(np.uint64)
        got_v = vout.cpu().numpy().view(np.uint32)
        assert np.array_equal(got_k, want_k), call
        assert np.array_equal(got_v, want_v), call
        # inputs untouched
        assert np.array_equal(kin.cpu().numpy().view(np.uint64), keys)


def test_sort_pairs_noalloc_unaligned_buffers(gbh_lib):
    # output buffers that start off a 16-byte boundary (views one element
    # into larger tensors) and a ragged last tile of odd length
    torch = pytest.importorskip("torch")
    stream = torch.cuda.current_stream()
    n = 3 * 4096 + 1001  # a ragged last tile of odd length
    keys, idx, want_k, want_v = _unsorted_and_sorted(n, 8)
    kin = torch.from_numpy(keys.view(np.int64)).cuda()
    vin = torch.from_numpy(idx.view(np.int32)).cuda()
    kout = torch.empty(n + 1, dtype=torch.int64, device="cuda")[1:]
    vout = torch.empty(n + 1, dtype=torch.int32, device="cuda")[1:]
    assert kout.data_ptr() % 16 and vout.data_ptr() % 16
    torch.cuda.synchronize()
    rc = gbh_lib.gbh_sort_pairs_noalloc(
        C.c_void_p(kin.data_ptr()), C.c_void_p(vin.data_ptr()), C.c_void_p(kout.data_ptr()),
        C.c_void_p(vout.data_ptr()), n, C.c_void_p(stream.cuda_stream))
    assert rc == abi.GBH_OK
    assert np.array_equal(kout.cpu().numpy().view(np.uint64), want_k)
    assert np.array_equal(vout.cpu().numpy().view(np.uint32), want_v)


def test_sort_pairs_noalloc_rejects_oversize(gbh_lib):
    rc = gbh_lib.gbh_sort_pairs_noalloc(C.c_void_p(1), C.c_void_p(1), C.c_void_p(1), C.c_void_p(1),
                                        (1 << 20) + 1, None)
    assert rc == abi.GBH_ERR_INVALID
