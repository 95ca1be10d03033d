"""Index checks of the kernels that consume index lists (compacted sample indices,
sparse-depth pixel lists): an index outside the declared row range is skipped
and raises the range bit of the device flag (read and cleared by
srf_read_device_flag) instead of touching memory -- the substitute for a
memory-checking tool on this path.  The out-of-range indices used here still
point inside the allocations (the buffers are allocated larger than the rows
declared to the kernels), so no access could fault even without the checks."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = 'cuda'


@pytest.fixture(scope='module', autouse=True)
def built():
    from simple_rf_gb300 import build as b
    b.build()


def _flag():
    from simple_rf_gb300 import _lib
    fl = ctypes.c_int(0)
    _lib.check(_lib.load().srf_read_device_flag(ctypes.byref(fl), None), 'flag')
    return fl.value


def test_row_gather_scatter_and_activation_skip_out_of_range_indices():
    from simple_rf_gb300 import _lib
    from simple_rf_gb300.functional import _ptr, _stream
    assert _flag() == 0
    rows, n, cols = 100, 8, 3
    src = torch.arange(2 * rows * cols, dtype=torch.float32, device=DEV).view(2 * rows, cols)   # 2x the declared rows
    idx = torch.tensor([0, 5, 99, 100, 150, 7, -1, 3], dtype=torch.int32, device=DEV)
    count = torch.tensor([n], dtype=torch.int32, device=DEV)
    dst = torch.full((n, cols), -7.0, device=DEV)
    _lib.call('srf_gather_rows', _ptr(dst), _ptr(src), rows, _ptr(idx), _ptr(count), n, cols, 1, _stream())
    torch.cuda.synchronize()
    good = np.array([True, True, True, False, False, True, False, True])
    ref = src.cpu().numpy()[np.clip(idx.cpu().numpy(), 0, None)]
    got = dst.cpu().numpy()
    np.testing.assert_array_equal(got[good], ref[good])
    assert (got[~good] == -7.0).all()
    assert _flag() & 1
    assert _flag() == 0   # read and cleared
    big = torch.zeros(2 * rows, cols, device=DEV)
    vals = torch.ones(n, cols, device=DEV)
    _lib.call('srf_scatter_rows', _ptr(big), rows, _ptr(vals), _ptr(idx), _ptr(count), n, cols, _stream())
    torch.cuda.synchronize()
    assert float(big[rows:].abs().sum()) == 0.0 and float(big[:rows].sum()) == 5 * cols
    assert _flag() & 1
    sig = torch.zeros(2 * rows, device=DEV)
    feat = torch.ones(n, device=DEV)
    _lib.call('srf_density_activation', _ptr(sig), rows, _ptr(feat), _ptr(idx), _ptr(count), n, 0, 0.0, _stream())
    torch.cuda.synchronize()
    assert float(sig[rows:].sum()) == 0.0 and float(sig[:rows].sum()) == 5.0
    assert _flag() & 1
    df = torch.full((n,), 3.0, device=DEV)
    _lib.call('srf_density_activation_backward', _ptr(df), _ptr(torch.ones(2 * rows, device=DEV)), rows, _ptr(feat),
              _ptr(idx), _ptr(count), n, 0, 0.0, _stream())
    torch.cuda.synchronize()
    np.testing.assert_array_equal(df.cpu().numpy(), np.where(good, 1.0, 0.0).astype(np.float32))
    assert _flag() & 1


def test_batch_assembly_flags_a_bad_pixel_list_entry():
    from simple_rf_gb300 import _lib
    from simple_rf_gb300.functional import _ptr, _stream
    assert _flag() == 0
    table = 50
    pid = torch.arange(3 * 2 * table, dtype=torch.int32, device=DEV).view(2 * table, 3)
    vals = torch.arange(2 * table, dtype=torch.float32, device=DEV).view(2 * table, 1)
    rows_list = torch.tensor([1, 2, 3, 60, 4, 5, 6, 7], dtype=torch.int32, device=DEV)   # 60 is past the table
    out_pid = torch.empty(8, 3, dtype=torch.int32, device=DEV)
    out_val = torch.empty(8, 1, device=DEV)
    out_idx = torch.empty(8, dtype=torch.int32, device=DEV)
    _lib.call('srf_batch_assemble', _ptr(rows_list), _ptr(pid), _ptr(vals), 1, 8, table, 8, 3, None, None, None, 0,
              _ptr(out_pid), _ptr(out_val), _ptr(out_idx), None, None, _stream())
    torch.cuda.synchronize()
    got = out_idx.cpu().numpy()
    assert (got < table).all() and sorted(set(got.tolist()) - {0}) == [1, 2, 3, 4, 5, 6, 7]
    assert _flag() & 1
