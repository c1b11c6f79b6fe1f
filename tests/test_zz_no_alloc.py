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
