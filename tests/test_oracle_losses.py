"""The loss oracle (oracle/losses.py) against the reference's own loss modules
(golden fixture tests/golden/losses.npz, made by tests/golden/make_golden.py)."""
import numpy as np

from oracle import losses as ol


def test_mass_concentration_matches_reference(golden):
    g = golden('losses')
    for s in (64, 67):
        loss, grad = ol.mass_concentration(g[f'mc{s}_weights'].astype(np.float64), 5, g['mask'])
        assert abs(loss - float(g[f'mc{s}_loss'])) < 1e-5 * abs(float(g[f'mc{s}_loss'])), s
        np.testing.assert_allclose(grad, g[f'mc{s}_grad'], rtol=1e-5, atol=1e-8)


def test_bin_sizes_follow_linspace_rule():
    # torch.linspace(0, 4, 4) = [0, 1.33, 2.67, 4] -> bins 0, 1, 2, 4 take the extra sample
    assert ol.bin_sizes(64, 5) == [13, 13, 13, 12, 13]
    for s, b in ((64, 5), (67, 5), (192, 7), (100, 10)):
        assert sum(ol.bin_sizes(s, b)) == s


def test_depth_losses_match_reference(golden):
    g = golden('losses')
    f64 = lambda k: g[k].astype(np.float64)  # noqa: E731
    loss, gp, _ = ol.depth_mse(f64('sd_pred'), f64('sd_true'), g['mask'], mean_over_mask=True)
    assert abs(loss - float(g['sd_loss'])) < 1e-5 * float(g['sd_loss'])
    np.testing.assert_allclose(gp, g['sd_grad'], rtol=1e-5, atol=1e-9)
    loss, gc, gf = ol.depth_mse(f64('cf_coarse'), f64('cf_fine'), target_grad=True)
    assert abs(loss - float(g['cf_loss'])) < 1e-5 * float(g['cf_loss'])
    np.testing.assert_allclose(gc, g['cf_grad_coarse'], rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(gf, g['cf_grad_fine'], rtol=1e-5, atol=1e-9)
    loss, gp, _ = ol.depth_mse(f64('ad_pred'), f64('ad_target'), g['mask'])
    assert abs(loss - float(g['ad_loss'])) < 1e-5 * float(g['ad_loss'])
    np.testing.assert_allclose(gp, g['ad_grad'], rtol=1e-5, atol=1e-9)


def test_reprojection_masks_and_loss_match_reference(golden):
    g = golden('reprojection')
    m1, m2, _, _ = ol.reprojection_masks(g['depth1'], g['depth2'], g['rays_o'], g['rays_d'], g['pixel_ids'],
                                         g['poses'], g['k'], g['images'], (5, 5), 0.2)
    np.testing.assert_array_equal(m1, g['mask1'])
    np.testing.assert_array_equal(m2, g['mask2'])
    assert m1.sum() > 10 and m2.sum() > 10
    loss, g1, g2 = ol.reprojection_depth_loss(g['depth1'].astype(np.float64), g['depth2'].astype(np.float64), m1, m2)
    assert abs(loss - float(g['loss'])) < 1e-5 * float(g['loss'])
    np.testing.assert_allclose(g1, g['grad1'], rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(g2, g['grad2'], rtol=1e-5, atol=1e-9)


def test_tv_loss_matches_reference(golden):
    g = golden('tv')
    w = float(g['iter_weight'])
    for tag in ('vm', 'cp'):
        comps = [g[f'{tag}_comp{i}'].astype(np.float64) for i in range(3)]
        loss, grads = ol.tv_loss(comps, w)
        assert abs(loss - float(g[f'{tag}_loss'])) < 1e-5 * abs(float(g[f'{tag}_loss'])), tag
        for i in range(3):
            np.testing.assert_allclose(grads[i], g[f'{tag}_grad{i}'], rtol=1e-5, atol=1e-9)
    assert abs(ol.tv_iter_weight(0.1, 30000, int(g['decay_iter_num'])) - float(g['decay_weight'])) < 1e-12


def test_tv_loss_single_row_and_column():
    # a (1, R, 1, 1) grid has no differences: loss 0, gradient 0 (counts floored at 1)
    loss, grads = ol.tv_loss([np.ones((1, 3, 1, 1))], 2.0)
    assert loss == 0.0 and not grads[0].any()


def test_coarse_fine_consistency_matches_reference(golden):
    """CoarseFineConsistencyLoss34.compute_loss (golden coarse_fine): masks on the NeRF
    rays without AugmentationsDepthLoss11's both-invalid rule (20 rays reproject
    outside the image with both depths), the masked depth term, the sparse-depth
    term, and the gradients into the coarse and fine depths."""
    g = golden('coarse_fine')
    loss, gc, gf, m1, m2 = ol.coarse_fine_consistency_loss(
        g['depth_coarse'].astype(np.float64), g['depth_fine'].astype(np.float64), g['nerf_mask'], g['sd_mask'],
        g['rays_o'], g['rays_d'], g['pixel_ids'], g['poses'], g['k'], g['images'], (5, 5), 0.2)
    np.testing.assert_array_equal(m1, g['mask1'])
    np.testing.assert_array_equal(m2, g['mask2'])
    assert abs(loss - float(g['loss'])) <= 1e-5 * abs(float(g['loss']))
    np.testing.assert_allclose(gc, g['grad_coarse'], rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(gf, g['grad_fine'], rtol=1e-5, atol=1e-9)
    # the rule AugmentationsDepthLoss11 adds would have selected rays here
    a1, a2, _, _ = ol.reprojection_masks(g['depth_coarse'][g['nerf_mask']], g['depth_fine'][g['nerf_mask']],
                                         g['rays_o'][g['nerf_mask']], g['rays_d'][g['nerf_mask']],
                                         g['pixel_ids'][g['nerf_mask']], g['poses'], g['k'], g['images'], (5, 5), 0.2)
    assert (a1 | a2).sum() > (m1 | m2).sum()
