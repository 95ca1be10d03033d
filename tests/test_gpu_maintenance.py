"""TensoRF grid-maintenance kernels against the torch CPU operators the reference
calls (SimpleTensoRF09.py:859-874 max_pool3d + threshold, :1284-1301
F.interpolate bilinear align_corners, :1303-1320 slicing), at the benchmark's
grid sizes: 300^2 planes with 16 / 48 components, 300-node lines, a 300^3
alpha volume.

Bars: pooling, threshold, the occupied range and cropping exact; resampling
within 1e-6 (torch's CPU kernel and the GPU round the same products and sums;
vectorised CPU paths may contract them)."""
import numpy as np
import pytest
import torch
import torch.nn.functional as tF

pytestmark = pytest.mark.gpu
DEV = 'cuda'


@pytest.fixture(scope='module', autouse=True)
def built():
    from simple_rf_gb300 import build as b
    b.build()


@pytest.mark.parametrize('shape', [(300, 300, 300), (33, 17, 9), (1, 1, 1), (2, 5, 1)])
def test_alpha_pool_threshold_matches_max_pool3d(shape):
    from simple_rf_gb300 import tensorf as T
    gx, gy, gz = shape
    g = torch.Generator().manual_seed(sum(shape))
    # a sparse field: most nodes far below the threshold, a few above
    alpha = torch.rand(gz, gy, gx, generator=g) ** 8 * 2e-4
    vol, rng = T.alpha_pool_threshold(alpha.to(DEV), 1e-4)
    ref = tF.max_pool3d(alpha[None, None], kernel_size=3, padding=1, stride=1)[0, 0]
    ref = (ref >= 1e-4).float()
    assert torch.equal(vol.cpu(), ref)
    occ = ref.nonzero()
    if occ.numel() == 0:
        assert rng is None
    else:
        lo = occ.amin(0).flip(0).tolist()   # (z, y, x) -> (x, y, z)
        hi = occ.amax(0).flip(0).tolist()
        assert rng == (tuple(lo), tuple(hi)), (rng, lo, hi)


def test_alpha_pool_threshold_empty_volume():
    from simple_rf_gb300 import tensorf as T
    vol, rng = T.alpha_pool_threshold(torch.zeros(4, 5, 6, device=DEV), 1e-4)
    assert rng is None and not vol.any()


@pytest.mark.parametrize('src,dst,comps', [((150, 150), (300, 300), 48), ((150, 150), (300, 300), 16),
                                           ((150, 1), (300, 1), 48), ((37, 23), (64, 41), 5), ((20, 30), (20, 30), 4),
                                           ((64, 64), (33, 17), 8), ((1, 7), (3, 9), 3)])
def test_resample_grid_matches_interpolate(src, dst, comps):
    from simple_rf_gb300 import tensorf as T
    g = torch.Generator().manual_seed(comps)
    x = torch.randn(1, comps, *src, generator=g) * 0.1
    got = T.resample_grid(T.to_channels_last(x.to(DEV)), *dst)
    ref = tF.interpolate(x, size=dst, mode='bilinear', align_corners=True)
    assert got.shape == ref.shape and got.is_contiguous(memory_format=torch.channels_last)
    np.testing.assert_allclose(got.cpu().numpy(), ref.numpy(), rtol=1e-6, atol=1e-6)


def test_crop_grid_matches_slicing():
    from simple_rf_gb300 import tensorf as T
    g = torch.Generator().manual_seed(1)
    x = torch.randn(1, 48, 300, 290, generator=g)
    got = T.crop_grid(T.to_channels_last(x.to(DEV)), 17, 281, 3, 250)
    assert torch.equal(got.cpu(), x[..., 17:281, 3:250])
    line = torch.randn(1, 16, 300, 1, generator=g)
    got = T.crop_grid(T.to_channels_last(line.to(DEV)), 40, 300, 0, 1)
    assert torch.equal(got.cpu(), line[..., 40:300, :])


def test_crop_grid_rejects_out_of_range_boxes():
    from simple_rf_gb300 import tensorf as T
    x = T.to_channels_last(torch.zeros(1, 4, 10, 10, device=DEV))
    for box in ((0, 11, 0, 10), (-1, 5, 0, 10), (0, 10, 5, 11)):
        with pytest.raises(RuntimeError):
            T.crop_grid(x, *box)


def test_alpha_grid_matches_reference_formula():
    """Dense alpha on the nodes of a 40 x 44 x 48 grid (R 16) against the same
    formula through the oracle's VM density (float64 reference evaluation of the
    nodes the reference forms from its CPU linspace, SimpleTensoRF09.py:849-858)."""
    from oracle import tensorf as ot
    from simple_rf_gb300 import tensorf as T
    res = [40, 44, 48]
    tp, _ = ot.seeded_vm_model(7, res, [16] * 3, [4] * 3, 7, 16)
    for kind in ('planes_density', 'lines_density'):
        tp[kind] = [a + np.float32(0.2) for a in tp[kind]]
    lo, hi = np.array([-1.5, -1.2, -1.0], np.float32), np.array([1.5, 1.3, 1.1], np.float32)
    grid = T.VmGridTensors.from_numpy(tp['planes_density'], tp['lines_density'], res, DEV)
    step = 0.03
    got = T.alpha_grid(grid, list(lo) + list(hi), None, None, step, 0, -10.0).cpu().numpy()
    s = [torch.linspace(0, 1, r).numpy() for r in res]
    xs, ys, zs = np.meshgrid(*s, indexing='ij')
    samples = np.stack([xs, ys, zs], -1).reshape(-1, 3).astype(np.float32)
    xyz = lo * (np.float32(1) - samples) + hi * samples
    pn = ot.normalize_points(xyz, np.stack([lo, hi]))
    sigma = np.maximum(ot.vm_density([p.astype(np.float64) for p in tp['planes_density']],
                                     [p.astype(np.float64) for p in tp['lines_density']], pn.astype(np.float64)), 0)
    ref = np.clip(1 - np.exp(-sigma * step), 0, 1).reshape(res).transpose(2, 1, 0)
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6)
    assert ref.max() > 0.01
