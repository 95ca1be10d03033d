"""Loss kernels (srf_depth_mse_loss, srf_mass_concentration_loss) against the
reference's own loss modules (golden fixture) and the loss oracle: loss values
and gradients within 1e-5 relative."""
import numpy as np
import pytest
import torch

from oracle import losses as ol

pytestmark = pytest.mark.gpu
DEV = 'cuda'


@pytest.fixture(scope='module', autouse=True)
def built():
    from simple_rf_gb300 import build as b
    b.build()


def _t(a, dtype=torch.float32):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV, dtype)


def _mass(weights, bins, mask):
    from simple_rf_gb300 import _lib
    from simple_rf_gb300.functional import _ptr, _stream
    w = _t(weights)
    m = _t(mask, torch.uint8) if mask is not None else None
    loss = torch.zeros(1, device=DEV)
    g = torch.zeros_like(w)
    _lib.call('srf_mass_concentration_loss', _ptr(w), w.shape[0], w.shape[1], bins, _ptr(m), 1.0, _ptr(loss),
              _ptr(g), _stream())
    torch.cuda.synchronize()
    return float(loss.item()), g.cpu().numpy()


def _depth(pred, target, mask, over_mask, both):
    from simple_rf_gb300 import _lib
    from simple_rf_gb300.functional import _ptr, _stream
    p, t = _t(pred), _t(target)
    m = _t(mask, torch.uint8) if mask is not None else None
    loss = torch.zeros(1, device=DEV)
    gp, gt = torch.zeros_like(p), torch.zeros_like(t)
    _lib.call('srf_depth_mse_loss', _ptr(p), _ptr(t), _ptr(m), p.shape[0], 1.0, int(over_mask), _ptr(loss), _ptr(gp),
              _ptr(gt) if both else None, _stream())
    torch.cuda.synchronize()
    return float(loss.item()), gp.cpu().numpy(), gt.cpu().numpy()


def test_mass_concentration_matches_reference_golden(golden):
    g = golden('losses')
    for s in (64, 67):
        loss, grad = _mass(g[f'mc{s}_weights'], 5, g['mask'])
        assert abs(loss - float(g[f'mc{s}_loss'])) < 1e-5 * abs(float(g[f'mc{s}_loss'])), s
        np.testing.assert_allclose(grad, g[f'mc{s}_grad'], rtol=1e-5, atol=1e-8)


def test_depth_losses_match_reference_golden(golden):
    g = golden('losses')
    loss, gp, _ = _depth(g['sd_pred'], g['sd_true'], g['mask'], True, False)
    assert abs(loss - float(g['sd_loss'])) < 1e-5 * float(g['sd_loss'])
    np.testing.assert_allclose(gp, g['sd_grad'], rtol=1e-5, atol=1e-9)
    loss, gc, gf = _depth(g['cf_coarse'], g['cf_fine'], None, False, True)
    assert abs(loss - float(g['cf_loss'])) < 1e-5 * float(g['cf_loss'])
    np.testing.assert_allclose(gc, g['cf_grad_coarse'], rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(gf, g['cf_grad_fine'], rtol=1e-5, atol=1e-9)
    loss, gp, _ = _depth(g['ad_pred'], g['ad_target'], g['mask'], False, False)
    assert abs(loss - float(g['ad_loss'])) < 1e-5 * float(g['ad_loss'])
    np.testing.assert_allclose(gp, g['ad_grad'], rtol=1e-5, atol=1e-9)


@pytest.mark.parametrize('n,s,bins', [(4096, 64, 5), (1000, 192, 7), (3, 10, 10), (0, 64, 5)])
def test_mass_concentration_against_oracle(n, s, bins):
    rng = np.random.default_rng(n + s)
    w = (rng.random((n, s)) * 0.03).astype(np.float32)
    mask = rng.random(n) < 0.8
    if n == 0:
        loss, grad = _mass(np.zeros((0, s), np.float32), bins, None)
        assert loss == 0.0 and grad.size == 0
        return
    ref_loss, ref_grad = ol.mass_concentration(w.astype(np.float64), bins, mask)
    loss, grad = _mass(w, bins, mask)
    assert abs(loss - ref_loss) < 1e-5 * abs(ref_loss), (loss, ref_loss)
    np.testing.assert_allclose(grad, ref_grad, rtol=1e-5, atol=1e-9)


def test_loss_kernels_reject_bad_shapes():
    from simple_rf_gb300 import _lib
    lib = _lib.load()
    w = torch.zeros(4, 8, device=DEV)
    assert lib.srf_mass_concentration_loss(w.data_ptr(), 4, 8, 9, None, 1.0, None, None, None) != 0   # bins > S
    assert lib.srf_mass_concentration_loss(w.data_ptr(), 4, 8, 65, None, 1.0, None, None, None) != 0
    assert lib.srf_depth_mse_loss(None, None, None, 4, 1.0, 0, None, None, None, None) != 0
    assert lib.srf_depth_mse_loss(None, None, None, 0, 1.0, 0, None, None, None, None) == 0


def _masks(g, thr=0.2):
    from simple_rf_gb300 import _lib
    from simple_rf_gb300.functional import _ptr, _stream
    n = g['depth1'].shape[0]
    t = {k: _t(g[k]) for k in ('rays_o', 'rays_d', 'depth1', 'depth2', 'poses', 'k', 'images')}
    pid = _t(g['pixel_ids'], torch.int32)
    m1 = torch.zeros(n, dtype=torch.uint8, device=DEV)
    m2 = torch.zeros_like(m1)
    v, h, w, c = g['images'].shape
    _lib.call('srf_depth_reprojection_masks', _ptr(t['rays_o']), _ptr(t['rays_d']), _ptr(t['depth1']),
              _ptr(t['depth2']), _ptr(pid), n, _ptr(t['poses']), v, _ptr(t['k']), _ptr(t['images']), h, w, c, 5, 5,
              thr, _ptr(m1), _ptr(m2), _stream())
    torch.cuda.synchronize()
    return m1.cpu().numpy().astype(bool), m2.cpu().numpy().astype(bool)


def test_reprojection_masks_match_reference_golden(golden):
    g = golden('reprojection')
    m1, m2 = _masks(g)
    np.testing.assert_array_equal(m1, g['mask1'])
    np.testing.assert_array_equal(m2, g['mask2'])


def test_reprojection_masks_against_oracle_random_scene():
    """4000 rays over 6 views with random rotations: masks equal the oracle's except
    on rays whose reprojection lies within 1e-3 px of a rounding boundary."""
    rng = np.random.default_rng(8)
    v, h, w = 6, 48, 64
    yy, xx = np.meshgrid(np.arange(h), np.arange(w), indexing='ij')
    base = np.stack([np.sin(xx / 6), np.cos(yy / 5), np.sin((xx + yy) / 9)], -1) * 0.5 + 0.5
    images = (0.9 * base[None] + 0.1 * rng.random((v, h, w, 3))).astype(np.float32)
    poses = np.tile(np.eye(4, dtype=np.float32), (v, 1, 1))
    for i in range(v):
        a = rng.normal(0, 0.03, 3)
        kx = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
        poses[i, :3, :3] = (np.eye(3) + kx + kx @ kx / 2).astype(np.float32)
        poses[i, :3, 3] = rng.uniform(-0.1, 0.1, 3)
    k = np.array([[40.0, 0, w / 2], [0, 40.0, h / 2], [0, 0, 1]], np.float32)
    n = 4000
    pid = np.stack([rng.integers(0, v, n), rng.integers(0, w, n), rng.integers(0, h, n)], 1).astype(np.int32)
    dirs = np.stack([(pid[:, 1] - w / 2) / 40.0, -(pid[:, 2] - h / 2) / 40.0, -np.ones(n)], 1)
    rays_d = np.einsum('nij,nj->ni', poses[pid[:, 0], :3, :3], dirs).astype(np.float32)
    rays_o = poses[pid[:, 0], :3, 3].astype(np.float32)
    g = dict(images=images, poses=poses, k=k, pixel_ids=pid, rays_o=rays_o, rays_d=rays_d,
             depth1=rng.uniform(1.0, 4.0, n).astype(np.float32), depth2=rng.uniform(1.0, 4.0, n).astype(np.float32))
    m1, m2 = _masks(g)
    r1, r2, p1, p2 = ol.reprojection_masks(g['depth1'], g['depth2'], rays_o, rays_d, pid, poses, k, images, (5, 5), 0.2)
    near = lambda p: (np.abs(np.abs(p - np.floor(p)) - 0.5) < 1e-3).any(1)  # noqa: E731
    bad = (m1 != r1) | (m2 != r2)
    assert r1.sum() > 100 and r2.sum() > 100
    assert not (bad & ~(near(p1) | near(p2))).any(), np.flatnonzero(bad)[:10]


def _tv_gpu(comps_np, weight, channels_last):
    from simple_rf_gb300 import functional as F
    ps = []
    for c in comps_np:
        p = _t(c)
        if channels_last:
            p = p.contiguous(memory_format=torch.channels_last)
        ps.append(p.requires_grad_(True))
    loss = F.tv_loss(ps, weight)
    loss.backward()
    torch.cuda.synchronize()
    return float(loss.item()), [p.grad.cpu().numpy() for p in ps], ps


@pytest.mark.parametrize('channels_last', [False, True])
def test_tv_loss_matches_reference_golden(golden, channels_last):
    g = golden('tv')
    w = float(g['iter_weight'])
    for tag in ('vm', 'cp'):
        comps = [g[f'{tag}_comp{i}'] for i in range(3)]
        loss, grads, ps = _tv_gpu(comps, w, channels_last)
        assert abs(loss - float(g[f'{tag}_loss'])) < 1e-5 * abs(float(g[f'{tag}_loss'])), tag
        for i in range(3):
            ref = g[f'{tag}_grad{i}']
            assert ps[i].grad.stride() == ps[i].stride()
            np.testing.assert_allclose(grads[i], ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())


def test_tv_loss_full_size_planes_against_oracle():
    # the three 300^2 x 48 colour planes of the 300^3 model, channels-last as the drop-in stores them
    gen = torch.Generator().manual_seed(5)
    comps = [(torch.randn(1, 48, 300, 300, generator=gen) * 0.1).numpy() for _ in range(3)]
    loss, grads, _ = _tv_gpu(comps, 0.25, True)
    ref_loss, ref_grads = ol.tv_loss([c.astype(np.float64) for c in comps], 0.25)
    assert abs(loss - ref_loss) < 1e-5 * abs(ref_loss)
    for a, b in zip(grads, ref_grads):
        np.testing.assert_allclose(a, b, rtol=1e-4, atol=1e-5 * np.abs(b).max())


def test_tv_loss_accumulate_adds_into_grad():
    from simple_rf_gb300 import functional as F
    gen = torch.Generator().manual_seed(6)
    comps = [torch.randn(1, 4, 13, 21, generator=gen) for _ in range(2)]
    ps = [c.to(DEV).contiguous(memory_format=torch.channels_last).requires_grad_(True) for c in comps]
    for p in ps:
        p.grad = torch.full_like(p, 0.5)
    loss = torch.zeros((), device=DEV)
    F.tv_loss_accumulate(ps, 3.0, loss)
    torch.cuda.synchronize()
    ref_loss, ref_grads = ol.tv_loss([c.numpy().astype(np.float64) for c in comps], 3.0)
    assert abs(float(loss.item()) - ref_loss) < 1e-5 * ref_loss
    for p, rg in zip(ps, ref_grads):
        np.testing.assert_allclose(p.grad.cpu().numpy(), rg + 0.5, rtol=1e-5, atol=1e-5 * np.abs(rg).max())


def test_tv_drop_in_loss_module_on_augmented_models():
    """TotalVariationLoss.compute_loss over a model's augmented VM (coarse) and CP
    (fine) grids: loss and parameter gradients against the oracle."""
    import types
    from simple_rf_gb300.bench_tensorf import tensor_configs, BBOX
    from simple_rf_gb300.losses import TotalVariationLoss
    from simple_rf_gb300.tensorf_model import make_tensor_model
    torch.manual_seed(3)
    cfg = {'data_loader': {'ndc': False}, 'model': {'white_bkgd': True}}
    vm = make_tensor_model('views_augmentation_coarse_model', cfg, tensor_configs(20 ** 3), {'bounding_box': BBOX})
    tc = dict(tensor_configs(16 ** 3), decomposition_type='CandecompParafac', num_components_density=[8],
              num_components_color=[24])
    cp = make_tensor_model('views_augmentation_fine_model', cfg, tc, {'bounding_box': BBOX})
    vm, cp = vm.to(DEV), cp.to(DEV)
    model = types.SimpleNamespace(module=types.SimpleNamespace(
        augmented_models=[{'name': 'views_augmentation', 'coarse_model': vm, 'fine_model': cp}]))
    configs = {'model': {'augmentations': [{'name': 'views_augmentation', 'coarse_model': {}, 'fine_model': {}}]},
               'num_iterations': 1000,
               'optimizers': [{'name': 'optimizer_main', 'lr_decay_ratio': 0.1, 'lr_decay_iters': None}]}
    tv = TotalVariationLoss(configs, {'weight_density': 0.5, 'weight_color': 0.25})
    loss = tv.compute_loss({'target_rgb': torch.zeros(1, 3, device=DEV), 'iter_num': 99}, {}, model)['loss_value']
    loss.backward()
    iw = ol.tv_iter_weight(0.1, 1000, 99)
    ref = 0.0
    for grids, w in ((vm.matrices_density, 0.5), (vm.matrices_color, 0.25), (cp.vectors_density, 0.5),
                     (cp.vectors_color, 0.25)):
        l, grads = ol.tv_loss([p.detach().cpu().numpy().astype(np.float64) for p in grids], iw * w)
        ref += l
        for p, rg in zip(grids, grads):
            np.testing.assert_allclose(p.grad.cpu().numpy(), rg, rtol=1e-5, atol=1e-5 * np.abs(rg).max())
    assert abs(float(loss.item()) - ref) < 1e-5 * ref


def test_tv_loss_rejects_bad_shapes():
    from simple_rf_gb300 import _lib
    lib = _lib.load()
    p = torch.zeros(1, 2, 3, 4, device=DEV)
    c = _lib.TvComponent(p.data_ptr(), None, 2, 3, 4, 1, 8, 2)
    arr = (_lib.TvComponent * 9)(*([c] * 9))
    assert lib.srf_tv_loss(arr, 9, 1.0, None, None, None) != 0                    # more than 8 components
    bad = (_lib.TvComponent * 1)(_lib.TvComponent(p.data_ptr(), None, 0, 3, 4, 1, 8, 2))
    assert lib.srf_tv_loss(bad, 1, 1.0, None, None, None) != 0                    # empty channel axis
    null = (_lib.TvComponent * 1)(_lib.TvComponent(None, None, 2, 3, 4, 1, 8, 2))
    assert lib.srf_tv_loss(null, 1, 1.0, None, None, None) != 0
    assert lib.srf_tv_loss(None, 0, 1.0, None, None, None) == 0


def _composite_setup(n, s, seed, white):
    from simple_rf_gb300 import _lib
    g = torch.Generator().manual_seed(seed)
    sigma = (torch.rand(n, s, generator=g) * 3 - 0.5).clamp_min(0).to(DEV)
    rgb = torch.rand(n, s, 3, generator=g).to(DEV)
    z = torch.sort(torch.rand(n, s, generator=g) * 4 + 2, 1).values.to(DEV).contiguous()
    d = torch.nn.functional.normalize(torch.randn(n, 3, generator=g), dim=-1).to(DEV)
    tr = torch.rand(n, 3, generator=g).to(DEV)
    td = (torch.rand(n, generator=g) * 4 + 2).to(DEV)
    dmask = (torch.rand(n, generator=g) < 0.25).to(torch.uint8).to(DEV)
    mcmask = (torch.rand(n, generator=g) < 0.6).to(torch.uint8).to(DEV)
    bufs = {k: torch.zeros(n, device=DEV) for k in ('acc', 'depth', 'depth_var')}
    bufs['rgb_map'] = torch.zeros(n, 3, device=DEV)
    bufs['weights'] = torch.zeros(n, s, device=DEV)
    a = _lib.CompositeArgs()
    a.n_rays, a.n_samples = n, s
    a.flags = _lib.SRF_COMPOSITE_WHITE_BKGD if white else 0
    a.distance_scale = 1.0
    a.sigma, a.rgb, a.z, a.rays_d = sigma.data_ptr(), rgb.data_ptr(), z.data_ptr(), d.data_ptr()
    a.rgb_map, a.acc, a.depth = bufs['rgb_map'].data_ptr(), bufs['acc'].data_ptr(), bufs['depth'].data_ptr()
    a.depth_var, a.weights = bufs['depth_var'].data_ptr(), bufs['weights'].data_ptr()
    keep = (sigma, rgb, z, d)
    return a, bufs, (tr, td, dmask, mcmask), keep


@pytest.mark.parametrize('s,white,bins,squared', [(192, True, 0, 0), (64, False, 5, 0), (256, True, 5, 1),
                                                  (129, False, 7, 0)])
def test_composite_fused_loss_matches_separate_kernels(s, white, bins, squared):
    """srf_composite_forward_loss / srf_composite_backward_loss (the training loss
    evaluated in the compositing epilogue, its gradient recomputed in the adjoint)
    against the separate path: srf_composite_forward, the loss kernels
    (srf_rgb_depth_loss for MSE14 + L1 depth, srf_depth_mse_loss for the squared
    depth error, srf_mass_concentration_loss for MassConcentrationLoss06), and
    srf_composite_backward fed with their gradients.  Loss within 1e-5 relative;
    d_sigma / d_rgb within 1e-6 relative (absolute floor 1e-9 of the range): the
    fused path sums each bin's weights in another order."""
    import ctypes
    from simple_rf_gb300 import _lib
    from simple_rf_gb300.functional import _stream
    n = 4096
    a, bufs, (tr, td, dmask, mcmask), keep = _composite_setup(n, s, 11 + s, white)
    st = _stream()
    nd, nmc = int(dmask.sum().item()), int(mcmask.sum().item())
    # separate kernels
    _lib.call('srf_composite_forward', ctypes.byref(a), st)
    loss_ref = torch.zeros(1, device=DEV)
    g_rgb = torch.zeros(n, 3, device=DEV)
    g_depth = torch.zeros(n, device=DEV)
    g_w = torch.zeros(n, s, device=DEV)
    if squared:
        _lib.call('srf_rgb_depth_loss', bufs['rgb_map'].data_ptr(), tr.data_ptr(), bufs['depth'].data_ptr(),
                  td.data_ptr(), None, n, 0, 0.0, loss_ref.data_ptr(), g_rgb.data_ptr(), g_depth.data_ptr(), st)
        _lib.call('srf_depth_mse_loss', bufs['depth'].data_ptr(), td.data_ptr(), dmask.data_ptr(), n, 0.1, 1,
                  loss_ref.data_ptr(), g_depth.data_ptr(), None, st)
    else:
        _lib.call('srf_rgb_depth_loss', bufs['rgb_map'].data_ptr(), tr.data_ptr(), bufs['depth'].data_ptr(),
                  td.data_ptr(), dmask.data_ptr(), n, nd, 0.1, loss_ref.data_ptr(), g_rgb.data_ptr(),
                  g_depth.data_ptr(), st)
    if bins:
        _lib.call('srf_mass_concentration_loss', bufs['weights'].data_ptr(), n, s, bins, mcmask.data_ptr(), 0.01,
                  loss_ref.data_ptr(), g_w.data_ptr(), st)
    ref_out = {k: v.clone() for k, v in bufs.items()}
    d_sigma_ref, d_rgb_ref = torch.zeros(n, s, device=DEV), torch.zeros(n, s, 3, device=DEV)
    a.g_rgb, a.g_depth = g_rgb.data_ptr(), g_depth.data_ptr()
    a.g_weights = g_w.data_ptr() if bins else None
    a.d_sigma, a.d_rgb = d_sigma_ref.data_ptr(), d_rgb_ref.data_ptr()
    _lib.call('srf_composite_backward', ctypes.byref(a), st)
    # fused
    for v in bufs.values():
        v.zero_()
    L = _lib.CompositeLoss()
    loss = torch.zeros(1, device=DEV)
    L.target_rgb, L.rgb_weight = tr.data_ptr(), 1.0
    L.target_depth, L.depth_mask, L.n_depth_rays, L.depth_weight, L.depth_squared = \
        td.data_ptr(), dmask.data_ptr(), nd, 0.1, squared
    if bins:
        L.num_bins, L.mc_mask, L.n_mc_rays, L.mc_weight = bins, mcmask.data_ptr(), nmc, 0.01
    L.loss = loss.data_ptr()
    a.g_rgb = a.g_depth = a.g_weights = None
    _lib.call('srf_composite_forward_loss', ctypes.byref(a), ctypes.byref(L), st)
    d_sigma, d_rgb = torch.zeros(n, s, device=DEV), torch.zeros(n, s, 3, device=DEV)
    a.d_sigma, a.d_rgb = d_sigma.data_ptr(), d_rgb.data_ptr()
    _lib.call('srf_composite_backward_loss', ctypes.byref(a), ctypes.byref(L), st)
    torch.cuda.synchronize()
    for k, v in bufs.items():
        assert torch.equal(v, ref_out[k]), k
    # the loss is a sum of per-ray terms added in another order: 1e-5 relative
    assert abs(loss.item() - loss_ref.item()) <= 1e-5 * abs(loss_ref.item()), (loss.item(), loss_ref.item())
    for got, ref, name in ((d_sigma, d_sigma_ref, 'd_sigma'), (d_rgb, d_rgb_ref, 'd_rgb')):
        np.testing.assert_allclose(got.cpu().numpy(), ref.cpu().numpy(), rtol=1e-6,
                                   atol=1e-9 * float(ref.abs().max().item()), err_msg=name)
    if not bins:
        assert torch.equal(d_sigma, d_sigma_ref) and torch.equal(d_rgb, d_rgb_ref)
    del keep


def test_composite_fused_loss_rejects_long_rays_and_bad_bins():
    import ctypes
    from simple_rf_gb300 import _lib
    from simple_rf_gb300.functional import _stream
    a, bufs, (tr, td, dmask, mcmask), keep = _composite_setup(64, 300, 1, False)
    L = _lib.CompositeLoss()
    loss = torch.zeros(1, device=DEV)
    L.target_rgb, L.loss = tr.data_ptr(), loss.data_ptr()
    lib = _lib.load()
    assert lib.srf_composite_forward_loss(ctypes.byref(a), ctypes.byref(L), _stream()) == \
        _lib.SRF_ERR_UNSUPPORTED
    a, bufs, (tr, td, dmask, mcmask), keep = _composite_setup(64, 64, 2, False)
    L.num_bins, L.n_mc_rays = 65, 64
    assert lib.srf_composite_forward_loss(ctypes.byref(a), ctypes.byref(L), _stream()) == _lib.SRF_ERR_SHAPE
    L.num_bins, L.loss = 5, None
    assert lib.srf_composite_forward_loss(ctypes.byref(a), ctypes.byref(L), _stream()) == _lib.SRF_ERR_NULL


def test_coarse_fine_consistency_drop_in_matches_reference_golden(golden):
    """The drop-in CoarseFineConsistencyLoss (srf_coarse_fine_reprojection_masks +
    srf_depth_mse_loss, autograd) against CoarseFineConsistencyLoss34.compute_loss
    (golden coarse_fine): loss and the gradients into the coarse and fine depths
    within 1e-5; the kernel's masks equal the reference's on the NeRF rays."""
    from simple_rf_gb300 import _lib
    from simple_rf_gb300.functional import _ptr, _stream
    from simple_rf_gb300.losses import CoarseFineConsistencyLoss
    g = golden('coarse_fine')
    nerf = g['nerf_mask']
    t = {k: _t(g[k]) for k in ('rays_o', 'rays_d', 'images', 'poses', 'k')}
    pid = _t(g['pixel_ids'], torch.int32)
    dc = _t(g['depth_coarse']).requires_grad_(True)
    df = _t(g['depth_fine']).requires_grad_(True)
    n = dc.shape[0]
    m1 = torch.empty(n, dtype=torch.uint8, device=DEV)
    m2 = torch.empty_like(m1)
    v, h, w, c = g['images'].shape
    _lib.call('srf_coarse_fine_reprojection_masks', _ptr(t['rays_o']), _ptr(t['rays_d']), _ptr(dc.detach()),
              _ptr(df.detach()), _ptr(pid), n, _ptr(t['poses']), v, _ptr(t['k']), _ptr(t['images']), h, w, c, 5, 5,
              0.2, _ptr(m1), _ptr(m2), _stream())
    np.testing.assert_array_equal(m1.cpu().numpy().astype(bool)[nerf], g['mask1'])
    np.testing.assert_array_equal(m2.cpu().numpy().astype(bool)[nerf], g['mask2'])
    configs = {'model': {'coarse_model': {}, 'fine_model': {}}, 'data_loader': {'sparse_depth': {}}}
    loss_fn = CoarseFineConsistencyLoss(configs, {'patch_size': [5, 5], 'rmse_threshold': 0.2})
    inp = {'target_rgb': torch.zeros(n, 3, device=DEV), 'pixel_id': pid,
           'common_data': {'images': t['images'], 'resolution': (h, w)},
           'indices_mask_nerf': torch.from_numpy(nerf).to(DEV),
           'indices_mask_sparse_depth': torch.from_numpy(g['sd_mask']).to(DEV)}
    out = {'rays_o': t['rays_o'], 'rays_d': t['rays_d'], 'depth_coarse': dc, 'depth_fine': df,
           'intrinsics': t['k'][None].repeat(n, 1, 1), 'extrinsics_all': t['poses']}
    loss = loss_fn.compute_loss(inp, out, None)['loss_value']
    loss.backward()
    assert abs(loss.item() - float(g['loss'])) <= 1e-5 * abs(float(g['loss']))
    np.testing.assert_allclose(dc.grad.cpu().numpy(), g['grad_coarse'], rtol=1e-5, atol=1e-8)
    np.testing.assert_allclose(df.grad.cpu().numpy(), g['grad_fine'], rtol=1e-5, atol=1e-8)


def test_augmentations_depth_drop_in_matches_reference_golden(golden):
    """The drop-in AugmentationsDepthLoss on the reprojection golden: the main depth
    as depth1, the augmented depth as depth2 (AugmentationsDepthLoss11.compute_loss_nerf),
    loss and gradients within 1e-5."""
    from simple_rf_gb300.losses import AugmentationsDepthLoss
    g = golden('reprojection')
    t = {k: _t(g[k]) for k in ('rays_o', 'rays_d', 'images', 'poses', 'k')}
    pid = _t(g['pixel_ids'], torch.int32)
    d1 = _t(g['depth1']).requires_grad_(True)
    d2 = _t(g['depth2']).requires_grad_(True)
    n = d1.shape[0]
    h, w = g['images'].shape[1:3]
    configs = {'model': {'coarse_model': {}, 'augmentations': [{'name': 'aug', 'coarse_model': {}}]}}
    loss_fn = AugmentationsDepthLoss(configs, {'patch_size': [5, 5], 'rmse_threshold': 0.2})
    inp = {'target_rgb': torch.zeros(n, 3, device=DEV), 'pixel_id': pid,
           'common_data': {'images': t['images'], 'resolution': (h, w)},
           'indices_mask_nerf': torch.ones(n, dtype=torch.bool, device=DEV)}
    out = {'rays_o': t['rays_o'], 'rays_d': t['rays_d'], 'depth_coarse': d1, 'aug_depth_coarse': d2,
           'intrinsics': t['k'][None].repeat(n, 1, 1), 'extrinsics_all': t['poses']}
    loss = loss_fn.compute_loss(inp, out, None)['loss_value']
    loss.backward()
    assert abs(loss.item() - float(g['loss'])) <= 1e-5 * abs(float(g['loss']))
    np.testing.assert_allclose(d1.grad.cpu().numpy(), g['grad1'], rtol=1e-5, atol=1e-8)
    np.testing.assert_allclose(d2.grad.cpu().numpy(), g['grad2'], rtol=1e-5, atol=1e-8)
