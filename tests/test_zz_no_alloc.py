"""The cell sort that allocates nothing (demsph_cell_sort_noalloc).

Callers that cannot allocate device memory at call time - their own allocator
already holds the GPU's memory, or they cannot afford cudaMalloc's device
synchronisation - use this entry point, whose scratch lives in a fixed device
array inside the library.  Its
result must equal the engine's own cell sort, read through the existing
entry point demsph_export_cell_hash, on two calls in a row (the array keeps
the previous call's contents, so the second call checks that whatever must
start at zero is cleared).  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 1 << 19


def _call(lib, keys, n, ncell, idx, cs, ce, stream):
    ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
    return lib.demsph_cell_sort_noalloc(ptr(keys), C.c_int(n), C.c_int(ncell), ptr(idx), ptr(cs), ptr(ce),
                                        C.c_void_p(stream))


@pytest.mark.parametrize("name", ("tiny_granular", "tiny_dam_break"))
def test_noalloc_sort_equals_engine_sort_on_two_calls(ds, scenes, name):
    import torch
    lib = ds.load_library()
    b, sc = ds.build_scene(getattr(scenes, name)())
    eng = ds.Engine(sc)
    eng.initialize()
    ref = eng.cell_hash(1)  # the engine's sort of the solids, through the existing C ABI
    n, ncell = sc.n_solid, eng.counts().grid_cells
    keys = np.empty(n, np.int32)
    keys[ref["index"]] = ref["value"]  # each particle's cell key, in original order
    dk = torch.from_numpy(keys).cuda()
    idx = torch.empty(n, dtype=torch.int32, device="cuda")
    cs = torch.empty(ncell, dtype=torch.int32, device="cuda")
    ce = torch.empty(ncell, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        for t in (idx, cs, ce):
            t.fill_(-7)
        assert _call(lib, dk, n, ncell, idx, cs, ce, stream) == 0, f"call {call}"
        assert np.array_equal(idx.cpu().numpy(), ref["index"]), f"call {call}: sorted index"
        assert np.array_equal(cs.cpu().numpy(), ref["start"]), f"call {call}: cell start"
        assert np.array_equal(ce.cpu().numpy(), ref["end"]), f"call {call}: cell end"


def test_noalloc_sort_large_keys_and_limits(ds):
    """The largest sizes (524,288 cells: the prefix sum at the one-block scan's
    limit) against a stable argsort, with every span checked; an empty call
    (n = 0, NULL keys and index) leaves every span empty; the limits and bad
    keys are rejected; and a good call after a rejected one is correct again
    (the array kept the rejected call's flag and counters)."""
    import torch
    lib = ds.load_library()
    rng = np.random.default_rng(7)
    n, ncell = 300_000, LIMIT
    keys = rng.integers(0, 20_000, size=n).astype(np.int32) * 17 % ncell
    order = np.argsort(keys, kind="stable").astype(np.int32)
    counts = np.bincount(keys, minlength=ncell)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    expect_start = np.where(counts > 0, starts, -1)
    expect_end = np.where(counts > 0, starts + counts, -1)
    dk = torch.from_numpy(keys).cuda()
    idx = torch.empty(n, dtype=torch.int32, device="cuda")
    cs = torch.empty(ncell, dtype=torch.int32, device="cuda")
    ce = torch.empty(ncell, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    def good_call(tag):
        for t in (idx, cs, ce):
            t.fill_(-7)
        assert _call(lib, dk, n, ncell, idx, cs, ce, stream) == 0, tag
        assert np.array_equal(idx.cpu().numpy(), order), tag
        assert np.array_equal(cs.cpu().numpy(), expect_start), tag
        assert np.array_equal(ce.cpu().numpy(), expect_end), tag

    for k in range(2):
        good_call(f"call {k}")
    cs.fill_(5)
    ce.fill_(5)
    assert _call(lib, None, 0, ncell, None, cs, ce, stream) == 0
    assert (cs.cpu().numpy() == -1).all() and (ce.cpu().numpy() == -1).all()
    assert _call(lib, dk, LIMIT + 1, ncell, idx, cs, ce, stream) == 1
    assert _call(lib, dk, n, LIMIT + 1, idx, cs, ce, stream) == 1
    bad = dk.clone()
    bad[5] = ncell
    assert _call(lib, bad, n, ncell, idx, cs, ce, stream) == 1
    good_call("after a rejected call")
