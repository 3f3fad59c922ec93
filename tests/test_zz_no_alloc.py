"""gbh_sort_pairs_noalloc, the sort entry point that allocates nothing.

It serves callers that cannot call cudaMalloc (device memory owned by another
allocator or engine, or a loop that must not touch the allocator).  The
expected result of every case is numpy's stable argsort of the keys, an
independent sort: keys and values after the call must equal keys[order] and
values[order] exactly (integer work, tolerance zero).  Cases:
  * the unsorted Morton keys and body indices of a step's compaction, also
    checked against the context's own sort stage (gbh_stage_sort), at the
    entry point's maximum size;
  * random 64-bit keys with the top bit set on half of them and many
    duplicates, so the last digit pass and the stability both matter;
  * buffers that start off a 16-byte boundary, with a ragged last tile;
  * an in-place sort (outputs identical to the inputs);
  * two calls in a row on the same scratch.

The file is named to be collected last, and it needs no other test's state.
"""
import ctypes as C

import numpy as np
import pytest

from gravity_gb300 import BarnesHut, abi, ic

pytestmark = pytest.mark.gpu


def _compaction_keys(n, seed):
    bodies = ic.plummer(n, seed=seed)
    sim = BarnesHut(n, ic.exact_bounds(bodies), abi.units(G=1.0))
    sim.upload_bodies(bodies)
    sim.init()
    p = abi.step_params()
    sim.reset_values(p)
    sim.partition_dead_bodies(p)  # compaction + bounds + Morton keys
    keys = sim.read_morton()[:n].copy()
    idx = sim.read_index()[:n].copy()
    sim.radix_sort()  # the context's own sort stage
    return keys, idx, sim.read_morton()[:n].copy(), sim.read_index()[:n].copy()


def _wide_keys(n, seed):
    rng = np.random.default_rng(seed)
    keys = rng.integers(0, 1 << 62, n, dtype=np.uint64) | (rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63))
    keys[rng.integers(0, n, n // 4)] = keys[rng.integers(0, n, n // 4)]  # duplicates
    return keys, rng.permutation(n).astype(np.uint32)


def _expected(keys, vals):
    order = np.argsort(keys, kind="stable")
    return keys[order], vals[order]


def _call(lib, torch, kin, vin, kout, vout, n):
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    return lib.gbh_sort_pairs_noalloc(
        C.c_void_p(kin.data_ptr()), C.c_void_p(vin.data_ptr()), C.c_void_p(kout.data_ptr()),
        C.c_void_p(vout.data_ptr()), n, C.c_void_p(stream.cuda_stream))


def _dev(torch, keys, vals):
    return torch.from_numpy(keys.view(np.int64)).cuda(), torch.from_numpy(vals.view(np.int32)).cuda()


def _host(kt, vt):
    return kt.cpu().numpy().view(np.uint64), vt.cpu().numpy().view(np.uint32)


def test_sort_pairs_noalloc_matches_stable_argsort(gbh_lib):
    torch = pytest.importorskip("torch")
    keys, idx, stage_k, stage_v = _compaction_keys(abi.SORT_NOALLOC_MAX_PAIRS, 6)
    want_k, want_v = _expected(keys, idx)
    assert np.array_equal(stage_k, want_k) and np.array_equal(stage_v, want_v)
    cases = [(keys, idx, want_k, want_v)]
    for n, seed in ((300000, 5), (4096 * 5 + 77, 9)):
        k, v = _wide_keys(n, seed)
        assert (k >> np.uint64(63)).any()
        cases.append((k, v) + _expected(k, v))
    for call, (k, v, wk, wv) in enumerate(cases):
        kin, vin = _dev(torch, k, v)
        kout, vout = torch.empty_like(kin), torch.empty_like(vin)
        # two calls in a row on the shared scratch give the same result
        for rep in range(2):
            kout.fill_(-1)
            vout.fill_(-1)
            assert _call(gbh_lib, torch, kin, vin, kout, vout, len(k)) == abi.GBH_OK, (call, rep)
            gk, gv = _host(kout, vout)
            assert np.array_equal(gk, wk), (call, rep)
            assert np.array_equal(gv, wv), (call, rep)
        ik, iv = _host(kin, vin)
        assert np.array_equal(ik, k) and np.array_equal(iv, v)  # inputs untouched


def test_sort_pairs_noalloc_in_place(gbh_lib):
    torch = pytest.importorskip("torch")
    k, v = _wide_keys(70001, 3)
    wk, wv = _expected(k, v)
    kt, vt = _dev(torch, k, v)
    assert _call(gbh_lib, torch, kt, vt, kt, vt, len(k)) == abi.GBH_OK
    gk, gv = _host(kt, vt)
    assert np.array_equal(gk, wk) and np.array_equal(gv, wv)


def test_sort_pairs_noalloc_unaligned_buffers(gbh_lib):
    # output buffers that start off a 16-byte boundary (views one element
    # into larger tensors) and a ragged last tile of odd length
    torch = pytest.importorskip("torch")
    n = 3 * 4096 + 1001
    k, v = _wide_keys(n, 8)
    wk, wv = _expected(k, v)
    kin, vin = _dev(torch, k, v)
    kout = torch.empty(n + 1, dtype=torch.int64, device="cuda")[1:]
    vout = torch.empty(n + 1, dtype=torch.int32, device="cuda")[1:]
    assert kout.data_ptr() % 16 and vout.data_ptr() % 16
    assert _call(gbh_lib, torch, kin, vin, kout, vout, n) == abi.GBH_OK
    gk, gv = _host(kout, vout)
    assert np.array_equal(gk, wk) and np.array_equal(gv, wv)


def test_sort_pairs_noalloc_rejects_bad_arguments(gbh_lib):
    torch = pytest.importorskip("torch")
    rc = gbh_lib.gbh_sort_pairs_noalloc(C.c_void_p(1), C.c_void_p(1), C.c_void_p(1), C.c_void_p(1),
                                        abi.SORT_NOALLOC_MAX_PAIRS + 1, None)
    assert rc == abi.GBH_ERR_INVALID
    # partly overlapping input and output
    buf = torch.zeros(2048, dtype=torch.int64, device="cuda")
    vals = torch.zeros(2048, dtype=torch.int32, device="cuda")
    rc = gbh_lib.gbh_sort_pairs_noalloc(C.c_void_p(buf.data_ptr()), C.c_void_p(vals.data_ptr()),
                                        C.c_void_p(buf[1:].data_ptr()), C.c_void_p(vals.data_ptr()), 1024, None)
    assert rc == abi.GBH_ERR_INVALID
