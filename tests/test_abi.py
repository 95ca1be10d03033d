"""The C-ABI library builds, loads and exports every symbol the header declares.

No compute is called here (there may be no GPU); these run in the CPU suite.
"""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, 'include', 'srf_gb300.h')


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(srf_[a-z0-9_]+)\s*\(', text)))


@pytest.fixture(scope='module')
def lib():
    from simple_rf_gb300 import build as b
    b.build()
    from simple_rf_gb300 import _lib
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from simple_rf_gb300 import _lib
    assert set(header_functions()) == set(_lib.exported_symbols())


def test_status_strings_and_version(lib):
    from simple_rf_gb300 import _lib
    assert lib.srf_version().decode().startswith('srf_gb300')
    for code in range(0, 9):
        assert lib.srf_status_string(code)
    assert b'NULL' in lib.srf_status_string(1)


def test_host_side_validation_without_gpu(lib):
    """Argument checks run on the host before any launch: NULLs and bad shapes
    return a status (never a crash), so callers get an error instead of a fault."""
    from simple_rf_gb300 import _lib
    assert lib.srf_stratified_z(None, None, 4, 8, 2.0, 6.0, 0, None) == 1
    assert lib.srf_stratified_z(ctypes.c_void_p(16), None, 4, 0, 2.0, 6.0, 0, None) == 2
    assert lib.srf_fine_z(ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), None, 4, 64, 2000, None) == 2
    assert lib.srf_composite_forward(None, None) == 1
    a = _lib.CompositeArgs()
    a.n_rays, a.n_samples = 4, 0
    a.sigma = a.z = a.rays_d = a.rgb = 16
    assert lib.srf_composite_forward(ctypes.byref(a), None) == 2
    g = _lib.VmGrid()
    assert lib.srf_vm_density_forward(ctypes.byref(g), None, 0, None, None) == 1
    assert lib.srf_compact(None, 10, None, None, None, 0, None) == 1


def test_mlp_fused_path_switch(lib):
    """The MLP forward-path switch is host state only: it round-trips, queries with a
    negative mode, and rejects modes above 2 with a negative status (apart from the
    modes it returns)."""
    prev = lib.srf_nerf_mlp_fused_path(-1)
    assert prev in (0, 1, 2)
    try:
        assert lib.srf_nerf_mlp_fused_path(0) == prev
        assert lib.srf_nerf_mlp_fused_path(2) == 0
        assert lib.srf_nerf_mlp_fused_path(-1) == 2
        assert lib.srf_nerf_mlp_fused_path(3) == -2
        assert lib.srf_nerf_mlp_fused_path(-1) == 2
    finally:
        lib.srf_nerf_mlp_fused_path(prev)
    assert lib.srf_nerf_mlp_fused_path(-1) == prev


def test_mlp_descriptor_and_workspace(lib):
    from simple_rf_gb300 import _lib
    d = _lib.NerfMlpDesc(8, 256, 1, 128, 10, 4, -1, 1, 1, 4)
    assert lib.srf_nerf_mlp_num_params(ctypes.byref(d)) == 24
    buf = ctypes.create_string_buffer(64)
    n = ctypes.c_int64()
    assert lib.srf_nerf_mlp_param_info(ctypes.byref(d), 10, buf, 64, ctypes.byref(n)) == 0
    assert buf.value == b'pts_linears.5.weight' and n.value == 256 * (256 + 63)
    ws_f = lib.srf_nerf_mlp_workspace_size(ctypes.byref(d), 1000, 0, 1)
    assert ws_f > 1000 * 256 * 4 * 8
    # the skip layer must leave room for a following layer
    bad = _lib.NerfMlpDesc(8, 256, 1, 128, 10, 4, -1, 1, 1, 7)
    assert lib.srf_nerf_mlp_workspace_size(ctypes.byref(bad), 1000, 0, 1) == 0
