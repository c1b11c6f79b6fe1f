"""The allocation-free block binning (si_block_sort_noalloc) against the library's own sort.

Callers that cannot allocate device memory (a host whose allocator owns the GPU's memory, a stream
being recorded into a graph, a frame loop that cannot stall on cudaFree) use this entry point; its
scratch is a fixed array inside the library. Two calls in a row, on two different particle states,
must give the keys, starts and order that si_mpm_sort gives (integers: exactly equal). This file is
collected last and also passes when run on its own."""
import ctypes

import numpy as np
import pytest

from shaderintel_gb300 import MPM
from shaderintel_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def reference_bins(sim):
    """keys, starts and order from the library's sort entry point (si_mpm_sort)."""
    before = sim.readParticles()
    sim._sort()
    keys, starts = sim.readBins()
    after = sim.readParticles()
    return before, keys, starts, after


def test_block_sort_noalloc_matches_sort_entry_point():
    torch = pytest.importorskip("torch")
    sim = MPM(grid=48, maxParticles=60000)
    sim.add({"box": [[0.1, 0.1, 0.1], [0.45, 0.5, 0.8]]}, material="water")
    sim.add({"sphere": [[0.7, 0.6, 0.5], 0.12]}, material="jelly", velocity=[0, -1, 0])
    n = sim.count
    assert 0 < n <= 262144
    dims = (ctypes.c_int32 * 3)(*sim.dims)
    nb = sim.numBlocks
    lib = L.lib()
    for call in range(2):                               # two calls in a row, two different states
        for _ in range(2 + 3 * call):
            sim.step()
        before, want_keys, want_starts, after = reference_bins(sim)
        x = torch.from_numpy(np.ascontiguousarray(before)).cuda()        # AoS records, stride 32
        keys = torch.empty(n, dtype=torch.int32, device="cuda")
        perm = torch.empty(n, dtype=torch.int32, device="cuda")
        starts = torch.empty(nb + 1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = lib.si_block_sort_noalloc(ctypes.cast(x.data_ptr(), L.c_float_p), 32, n, dims,
                                       ctypes.cast(keys.data_ptr(), L.c_uint32_p),
                                       ctypes.cast(perm.data_ptr(), L.c_uint32_p),
                                       ctypes.cast(starts.data_ptr(), L.c_uint32_p), None)
        L.check(rc)
        torch.cuda.synchronize()
        got_keys = keys.cpu().numpy().view(np.uint32)
        got_perm = perm.cpu().numpy().view(np.uint32)
        got_starts = starts.cpu().numpy().view(np.uint32)
        assert np.array_equal(got_keys, want_keys), f"call {call}: keys differ"
        assert np.array_equal(got_starts, want_starts), f"call {call}: starts differ"
        assert np.array_equal(before[got_perm].view(np.uint32), after.view(np.uint32)), f"call {call}: order differs"
    sim.destroy()


def test_block_sort_noalloc_rejects_too_many_particles():
    dims = (ctypes.c_int32 * 3)(64, 64, 64)
    one = (ctypes.c_uint32 * 1)()
    x = (ctypes.c_float * 4)()
    rc = L.lib().si_block_sort_noalloc(x, 4, 262145, dims, one, one, one, None)
    assert rc == L.SI_EINVAL
    assert b"262144" in L.lib().si_last_error()


def _noalloc(x_t, stride, n, dims, nb, stream=None):
    """One call through the C ABI on device tensors; returns keys, perm, starts as numpy uint32."""
    import torch
    keys = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    perm = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    starts = torch.full((nb + 1,), -1, dtype=torch.int32, device="cuda")
    d = (ctypes.c_int32 * 3)(*dims)
    torch.cuda.synchronize()
    rc = L.lib().si_block_sort_noalloc(ctypes.cast(x_t.data_ptr(), L.c_float_p), stride, n, d,
                                       ctypes.cast(keys.data_ptr(), L.c_uint32_p),
                                       ctypes.cast(perm.data_ptr(), L.c_uint32_p),
                                       ctypes.cast(starts.data_ptr(), L.c_uint32_p),
                                       None if stream is None else ctypes.c_void_p(stream.cuda_stream))
    L.check(rc)
    (stream or torch.cuda.current_stream()).synchronize()
    torch.cuda.synchronize()
    return (keys.cpu().numpy().view(np.uint32)[:n], perm.cpu().numpy().view(np.uint32)[:n],
            starts.cpu().numpy().view(np.uint32))


def _expected(xyz, dims):
    """keys from the oracle, the stable order of those keys, and the block starts (lower bounds)."""
    import si_oracle as O
    nb = O.num_blocks(dims)
    rec = np.zeros((len(xyz), 32), np.float32)
    rec[:, :3] = xyz
    k = O.keys(rec, nb) if len(xyz) else np.zeros(0, np.uint32)
    order = np.argsort(k, kind="stable").astype(np.uint32)
    starts = np.searchsorted(k[order], np.arange(nb + 1, dtype=np.uint32), side="left").astype(np.uint32)
    return nb, k, order, starts


@pytest.mark.parametrize("case", ["empty", "cap_stride3_stream", "stride4_twice"])
def test_block_sort_noalloc_edge_cases(case):
    """n = 0 (all starts zero), n at the 262144 cap with packed xyz (stride 3) on a non-default
    stream, and a stride-4 input sorted twice in a row: keys, order and starts equal the oracle's
    keys with a stable argsort of them."""
    torch = pytest.importorskip("torch")
    dims = (64, 64, 64)
    rng = np.random.default_rng(7)
    if case == "empty":
        nb, _, _, want_starts = _expected(np.zeros((0, 3), np.float32), dims)
        x = torch.zeros(4, dtype=torch.float32, device="cuda")
        keys, perm, starts = _noalloc(x, 3, 0, dims, nb)
        assert np.array_equal(starts, np.zeros(nb + 1, np.uint32))
        return
    if case == "cap_stride3_stream":
        n = 262144
        xyz = rng.uniform(2.0, 62.0, (n, 3)).astype(np.float32)
        nb, want_k, want_o, want_s = _expected(xyz, dims)
        x = torch.from_numpy(np.ascontiguousarray(xyz).reshape(-1)).cuda()
        s = torch.cuda.Stream()
        keys, perm, starts = _noalloc(x, 3, n, dims, nb, stream=s)
        assert np.array_equal(keys, want_k) and np.array_equal(perm, want_o) and np.array_equal(starts, want_s)
        return
    n = 50000
    for call in range(2):
        xyz = rng.uniform(0.0, 64.0, (n, 3)).astype(np.float32)
        xyz[: n // 10] = xyz[0]                          # a crowded block as well
        nb, want_k, want_o, want_s = _expected(xyz, dims)
        rec4 = np.zeros((n, 4), np.float32)
        rec4[:, :3] = xyz
        x = torch.from_numpy(rec4.reshape(-1)).cuda()
        keys, perm, starts = _noalloc(x, 4, n, dims, nb)
        assert np.array_equal(keys, want_k), f"call {call}: keys"
        assert np.array_equal(perm, want_o), f"call {call}: order"
        assert np.array_equal(starts, want_s), f"call {call}: starts"
