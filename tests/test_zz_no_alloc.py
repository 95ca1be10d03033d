"""srf_compact_noalloc: compaction for callers that cannot allocate device memory.

Such callers (a plugin living inside another framework's fixed memory pool, a
loop holding a no-allocation guarantee, a binding that only holds the mask and
output pointers) cannot hand srf_compact its scratch buffer; this entry point
keeps its scratch in a fixed array inside the library instead.  The test calls
it through the C ABI twice in a row (the second call must not see the first
call's leftovers in the shared array) and checks each result against the
existing srf_compact entry point: indices and counts are integers, so they
must match exactly.  It runs alone in a fresh process as well as after the
rest of the suite.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _with_workspace(lib, mask):
    n = mask.numel()
    idx = torch.full((n,), -1, dtype=torch.int32, device='cuda')
    cnt = torch.zeros(1, dtype=torch.int32, device='cuda')
    ws = torch.empty(lib.srf_compact_workspace_size(n), dtype=torch.uint8, device='cuda')
    assert lib.srf_compact(_p(mask), n, _p(idx), _p(cnt), _p(ws), ws.numel(), _stream()) == 0
    return idx, cnt


def _no_alloc(lib, mask):
    n = mask.numel()
    idx = torch.full((n,), -1, dtype=torch.int32, device='cuda')
    cnt = torch.zeros(1, dtype=torch.int32, device='cuda')
    assert lib.srf_compact_noalloc(_p(mask), n, _p(idx), _p(cnt), _stream()) == 0
    return idx, cnt


def test_noalloc_compaction_matches_workspace_version_twice():
    from simple_rf_gb300 import build as b
    b.build()
    from simple_rf_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(123)
    # a large dense mask first, then a smaller sparse one: the second call reads
    # only scratch it rewrote itself, whatever the first call left behind
    masks = [rng.random(3_000_001) < 0.6, rng.random(777_777) < 0.05]
    for m in masks:
        mask = torch.from_numpy(m.astype(np.uint8)).cuda()
        ref_idx, ref_cnt = _with_workspace(lib, mask)
        idx, cnt = _no_alloc(lib, mask)
        torch.cuda.synchronize()
        c = int(ref_cnt.item())
        assert c == int(np.count_nonzero(m))
        assert int(cnt.item()) == c
        assert torch.equal(idx[:c], ref_idx[:c])


def test_noalloc_compaction_at_the_size_limit_and_empty():
    """A mask of exactly the largest accepted size (every scratch slot in use) and
    an empty mask (the count is reset to 0 without a compaction launch)."""
    from simple_rf_gb300 import _lib
    lib = _lib.load()
    limit = 16384 * 1024
    rng = np.random.default_rng(7)
    m = rng.random(limit) < 0.3
    mask = torch.from_numpy(m.astype(np.uint8)).cuda()
    ref_idx, ref_cnt = _with_workspace(lib, mask)
    idx, cnt = _no_alloc(lib, mask)
    torch.cuda.synchronize()
    c = int(ref_cnt.item())
    assert c == int(np.count_nonzero(m)) and int(cnt.item()) == c
    assert torch.equal(idx[:c], ref_idx[:c])
    cnt = torch.full((1,), 12345, dtype=torch.int32, device='cuda')
    one = torch.zeros(1, dtype=torch.uint8, device='cuda')
    out = torch.zeros(1, dtype=torch.int32, device='cuda')
    assert lib.srf_compact_noalloc(_p(one), 0, _p(out), _p(cnt), _stream()) == 0
    torch.cuda.synchronize()
    assert int(cnt.item()) == 0


def test_noalloc_compaction_rejects_oversized_masks():
    from simple_rf_gb300 import _lib
    lib = _lib.load()
    limit = 16384 * 1024
    one = torch.zeros(1, dtype=torch.uint8, device='cuda')
    out = torch.zeros(1, dtype=torch.int32, device='cuda')
    # checked on the host before any launch: the pointers are never touched
    assert lib.srf_compact_noalloc(_p(one), limit + 1, _p(out), _p(out), _stream()) == 2
    assert lib.srf_compact_noalloc(None, 10, _p(out), _p(out), _stream()) == 1
