"""The numpy oracle against golden vectors produced by the reference's own code.

These pin the oracle (``oracle/``) before any CUDA result is compared with it.
Tolerances: float32 restatement vs torch-CPU float32; differences come only from
summation order and libm rounding, so 1e-5 relative (with a small absolute floor
for values near zero) is the bar, the same as the CUDA plain-path bar.
"""
import numpy as np
import pytest

from oracle import nerf as on
from oracle import tensorf as ot

RTOL, ATOL = 1e-5, 1e-6


def close(a, b, rtol=RTOL, atol=ATOL):
    np.testing.assert_allclose(np.asarray(a, np.float64), np.asarray(b, np.float64), rtol=rtol, atol=atol)


def cdf_of(bins, weights, x):
    """Piecewise-linear CDF of the reference's pdf (weights + 1e-5) evaluated at x, per row."""
    w = weights.astype(np.float64) + 1e-5
    cdf = np.concatenate([np.zeros((w.shape[0], 1)), np.cumsum(w / w.sum(-1, keepdims=True), -1)], -1)
    return np.stack([np.interp(x[r], bins[r].astype(np.float64), cdf[r]) for r in range(x.shape[0])])


def close_pdf(bins, weights, got, ref, tol=1e-5):
    """Inverse-CDF samples agree when they map to the same CDF value.

    sample_pdf (SimpleNeRF17.py:384-417) divides by cdf differences as small as
    1e-5, so a one-ulp change of ``sum(weights)`` (torch's float32 sum rounds
    differently per host SIMD width) moves a sample by up to ~1e-3 relative in z
    where the pdf is small, and can flip the bin at a ``denom < 1e-5`` step.  In
    CDF space both effects stay below the reference's own pdf floor of 1e-5.
    """
    d = np.abs(cdf_of(bins, weights, got) - cdf_of(bins, weights, ref))
    assert d.max() < tol, d.max()
    assert np.mean(~np.isclose(got, ref, rtol=2e-6, atol=2e-6)) < 0.01


def test_linspace_matches_reference_formula():
    for steps in (1, 2, 3, 64, 127, 128, 1039):
        x = on.torch_linspace(0., 1., steps)
        assert x[0] == 0.0 and (steps == 1 or x[-1] == 1.0)
        assert np.all(np.diff(x) >= 0)


def test_stratified_and_pdf_sampling(golden):
    g = golden('nerf_sampling')
    n, sc = g['u_coarse'].shape
    # torch.linspace rounds its vectorised second half differently per host SIMD
    # width, so the sample positions agree to one float32 ulp, not bit for bit.
    zc = on.stratified_z(2.0, 6.0, n, sc, g['u_coarse'])
    close(zc, g['z_coarse'], rtol=2.5e-7, atol=0)
    close(on.stratified_z(2.0, 6.0, n, sc, None), g['z_coarse_det'], rtol=2.5e-7, atol=0)
    zc = g['z_coarse']
    mids = np.float32(.5) * (zc[:, 1:] + zc[:, :-1])
    sf = g['u_fine'].shape[1]
    w = g['weights'][:, 1:-1]
    s = on.sample_pdf(mids, w, sf, g['u_fine'])
    close_pdf(mids, w, s, g['samples'])
    close_pdf(mids, w, on.sample_pdf(mids, w, sf, None), g['samples_det'])
    # the merged/sorted z: compare as multisets row by row (a flipped sample moves
    # within its row's sorted order)
    for u, key in ((g['u_fine'], 'z_fine'), (None, 'z_fine_det')):
        zf = on.fine_z(zc, g['weights'], sf, u)
        bad = ~np.isclose(zf, g[key], rtol=2e-6, atol=2e-6)
        assert bad.mean() < 0.01, key


def test_positional_encoding(golden):
    g = golden('nerf_pe')
    for deg in (10, 4, 3, 2, 0):
        close(on.positional_encoding(g['x'], deg), g[f'pe{deg}'], rtol=1e-6, atol=2e-6)


def test_mlp_variants(golden):
    g = golden('nerf_mlp')
    variants = {
        'main': on.MlpSpec(),
        'aug_l4_noview': on.MlpSpec(points_pe_degree=4, use_view_dirs=False, view_dependent_rgb=False),
        'points_aug': on.MlpSpec(points_sigma_pe_degree=3),
    }
    for i, (name, spec) in enumerate(variants.items()):
        p = on.xavier_params(spec, 1000 + i)
        sigma, rgb, _ = on.mlp_forward(p, spec, g['pts'], g['vdirs'])
        close(sigma, g[f'{name}_sigma'], rtol=1e-4, atol=1e-5)
        close(rgb, g[f'{name}_rgb'], rtol=1e-5, atol=1e-6)


def test_mac_counts():
    assert on.MlpSpec().macs_per_sample() == 593408
    assert on.MlpSpec(points_pe_degree=4, use_view_dirs=False, view_dependent_rgb=False).macs_per_sample() == 473600


@pytest.mark.parametrize('tag', ['world', 'ndc'])
def test_composite_forward_backward(golden, tag):
    g = golden('nerf_composite')
    ndc = tag == 'ndc'
    kw = dict(ndc=ndc, white_bkgd=True)
    if ndc:
        kw.update(rays_o=g[f'{tag}_rays_o'], rays_d_ndc=g[f'{tag}_rays_d_ndc'])
    out, cache = on.composite_forward(g[f'{tag}_sigma'], g[f'{tag}_rgb'], g[f'{tag}_z'], g[f'{tag}_rays_d'], **kw)
    for k, v in out.items():
        close(v, g[f'{tag}_out_{k}'], rtol=2e-5, atol=2e-6)
    cot = {k: g[f'{tag}_cot_{k}'] for k in out if k not in ('alpha', 'visibility')}
    dsig, drgb = on.composite_backward(cache, cot)
    ref = g[f'{tag}_dsigma']
    scale = np.abs(ref).max()
    close(dsig, ref, rtol=1e-4, atol=1e-5 * scale)
    close(drgb, g[f'{tag}_drgb'], rtol=1e-5, atol=1e-6)


def test_rays(golden):
    g = golden('rays')
    o, d = on.rays_from_pixels(g['pixel_id'], g['intrinsics'], g['extrinsics'])
    close(o, g['rays_o'])
    close(d, g['rays_d'])
    o2, d2 = on.rays_from_pixels(g['pixel_id'], g['intrinsics'], g['extrinsics'], half_pixel=True)
    close(d2, g['rays_d_half'])
    f = g['intrinsics'][:, 0, 0]
    on_, dn = on.ndc_rays(o, d, 378, 504, f, g['intrinsics'][:, 1, 1], 1.0)
    close(on_, g['rays_o_ndc'], rtol=1e-5, atol=1e-5)
    close(dn, g['rays_d_ndc'], rtol=1e-5, atol=1e-5)
    close(on.view_dirs(d), g['view_dirs'])


def _render(g, sc, sf, width=256, wv=128, white=False, ndc=False, aug=None):
    spec = on.MlpSpec(points_net_width=width, views_net_width=wv)
    seed = int(g['seed'])
    pc, pf = on.xavier_params(spec, seed), on.xavier_params(spec, seed + 1)
    nd = None
    if ndc:
        n = g['rays_o'].shape[0]
        f = np.full(n, g['focal'], np.float32)
        nd = dict(h=378, w=504, fx=f, fy=f, near=1.0)
    near, far = (0.0, 1.0) if ndc else (2.0, 6.0)
    return on.render_rays(pc, pf, spec, spec, g['rays_o'], g['rays_d'], near, far, sc, sf, g['u_coarse'],
                          g['u_fine'], white_bkgd=white, ndc=nd, aug=aug), (pc, pf, spec)


def _check_render(ret, g, keys_exact, keys_fine):
    """Coarse outputs at 1e-4 relative; fine z in CDF space (sample_pdf conditioning,
    see :func:`close_pdf`); fine per-ray outputs at 1e-4 relative of their range."""
    for k in keys_exact:
        ref = g['out_' + k]
        close(ret[k], ref, rtol=1e-4, atol=1e-5 * max(1.0, float(np.abs(ref).max())))
    zc = g['out_z_vals_coarse']
    mids = .5 * (zc[:, 1:] + zc[:, :-1])
    w = g['out_weights_coarse'][:, 1:-1]
    # the oracle builds its pdf from its own coarse weights (equal to 1e-5
    # relative), so the CDF-space bar here is 3e-5 rather than the sampler's 1e-5
    d = np.abs(cdf_of(mids, w, ret['z_vals_fine']) - cdf_of(mids, w, g['out_z_vals_fine']))
    assert d.max() < 3e-5, d.max()
    for k in keys_fine:
        ref = g['out_' + k]
        close(ret[k], ref, rtol=1e-4, atol=1e-4 * max(1.0, float(np.abs(ref).max())))


def test_render_config1_small(golden):
    g = golden('nerf_render')
    (ret, _), _ = _render(g, 64, 128)
    _check_render(ret, g, ('z_vals_coarse', 'rgb_coarse', 'weights_coarse', 'depth_coarse', 'acc_coarse'),
                  ('rgb_fine', 'acc_fine', 'depth_fine', 'depth_var_fine'))


def test_render_ndc_pair(golden):
    g = golden('nerf_ndc_pair')
    aspec = on.MlpSpec(points_pe_degree=4, use_view_dirs=False, view_dependent_rgb=False)
    aug = [('views_augmentation', {'coarse': on.xavier_params(aspec, 77)}, aspec)]
    (ret, _), _ = _render(g, 64, 128, ndc=True, aug=aug)
    _check_render(ret, g, ('rgb_coarse', 'depth_coarse', 'depth_ndc_coarse', 'weights_coarse',
                           'views_augmentation_rgb_coarse', 'views_augmentation_depth_coarse',
                           'views_augmentation_weights_coarse'),
                  ('rgb_fine', 'depth_ndc_fine', 'depth_fine', 'acc_fine'))


def test_train_step_gradients(golden):
    g = golden('nerf_train_grads')
    (ret, caches), (pc, pf, spec) = _render(g, 16, 32, width=32, wv=16, white=True)
    loss, grads = on.train_loss(ret, g['t_rgb'], g['t_depth'], g['dmask'])
    assert abs(loss - float(g['loss'])) < 1e-5 * max(1, abs(float(g['loss'])))
    pg = on.backward_render({'coarse': pc, 'fine': pf}, {'coarse': spec, 'fine': spec}, caches, grads,
                            g['rays_o'].shape[0])
    for tag in ('coarse', 'fine'):
        for k, v in pg[tag].items():
            ref = g[f'grad_{tag}.{k}']
            err = np.linalg.norm(v - ref) / max(np.linalg.norm(ref), 1e-12)
            assert err < 1e-4, (tag, k, err)


def _tensorf_params(g):
    tp = {'bbox': g['bbox']}
    for kind in ('planes_density', 'lines_density', 'planes_color', 'lines_color'):
        tp[kind] = [g[f'{kind}.{i}'] for i in range(3)]
    for k in g:
        if k.startswith('color_predictor.') or k == 'basis_matrix_color.weight':
            tp[k] = g[k]
    return tp


def test_tensorf_forward_backward(golden):
    g = golden('tensorf')
    tp = _tensorf_params(g)
    spec = ot.RendererSpec(features_dim=7, features_pe=2, views_pe=2, units=16)
    n = g['rays_o'].shape[0]
    z = ot.aabb_z(g['rays_o'], g['rays_d'], g['bbox'], 0.5, 6.0, float(g['step_size']), int(g['num_samples']), g['u'])
    close(z, g['z'], rtol=1e-6, atol=1e-6)
    out, cache = ot.tensorf_forward(tp, spec, g['rays_o'], g['rays_d'], g['z'], alpha_vol=g['alpha_vol'],
                                    alpha_bbox=g['bbox'], white=True)
    for k in ('rgb', 'depth', 'acc', 'weights', 'raw_sigma', 'raw_rgb', 'depth_var'):
        ref = g['out_' + k]
        close(out[k], ref, rtol=1e-5, atol=1e-6 * max(1.0, float(np.abs(ref).max())))
    assert n == out['rgb'].shape[0]
    grads = ot.tensorf_backward(tp, spec, cache, {k: g[f'cot_{k}'] for k in ('rgb', 'depth', 'acc')})
    for k, v in grads.items():
        ref = g['grad_' + k]
        err = np.linalg.norm(v - ref) / max(np.linalg.norm(ref), 1e-12)
        assert err < 1e-5, (k, err)


def test_tensorf_ndc_forward_backward(golden):
    """The oracle's NDC path against LowRankTensor.forward in NDC mode (golden
    tensorf_ndc): stratified NDC depths, NDC marching, metric depth conversion."""
    g = golden('tensorf_ndc')
    tp = _tensorf_params(g)
    spec = ot.RendererSpec(features_dim=7, features_pe=2, views_pe=2, units=16)
    n, s = g['z'].shape
    close(on.stratified_z(0.0, 1.0, n, s, g['u']), g['z'], rtol=1e-6, atol=1e-7)
    out, cache = ot.tensorf_forward(tp, spec, g['rays_o_ndc'], g['rays_d_ndc'], g['z'], alpha_vol=g['alpha_vol'],
                                    alpha_bbox=g['bbox'], white=False, world_rays=(g['rays_o'], g['rays_d']))
    for k in ('rgb', 'depth', 'depth_ndc', 'acc', 'weights', 'raw_sigma', 'raw_rgb', 'depth_var', 'depth_var_ndc'):
        ref = g['out_' + k]
        close(out[k], ref, rtol=1e-5, atol=1e-6 * max(1.0, float(np.abs(ref).max())))
    grads = ot.tensorf_backward(tp, spec, cache, {k: g[f'cot_{k}'] for k in ('rgb', 'depth', 'depth_ndc', 'acc')})
    for k, v in grads.items():
        ref = g['grad_' + k]
        err = np.linalg.norm(v - ref) / max(np.linalg.norm(ref), 1e-12)
        assert err < 1e-5, (k, err)


def test_tensorf_cp_forward_backward(golden):
    """The oracle's CP path against CpDecomposedTensor (golden tensorf_cp)."""
    g = golden('tensorf_cp')
    tp = {'bbox': g['bbox']}
    for kind in ('lines_density', 'lines_color'):
        tp[kind] = [g[f'{kind}.{i}'] for i in range(3)]
    for k in g:
        if k.startswith('color_predictor.') or k == 'basis_matrix_color.weight':
            tp[k] = g[k]
    spec = ot.RendererSpec(features_dim=7, features_pe=2, views_pe=2, units=16)
    out, cache = ot.tensorf_forward(tp, spec, g['rays_o'], g['rays_d'], g['z'], white=True)
    for k in ('rgb', 'depth', 'acc', 'weights', 'raw_sigma', 'raw_rgb', 'depth_var'):
        ref = g['out_' + k]
        close(out[k], ref, rtol=1e-5, atol=1e-6 * max(1.0, float(np.abs(ref).max())))
    grads = ot.tensorf_backward(tp, spec, cache, {k: g[f'cot_{k}'] for k in ('rgb', 'depth', 'acc')})
    assert set(grads) >= {'lines_density.0', 'lines_color.2', 'basis_matrix_color.weight'}
    for k, v in grads.items():
        ref = g['grad_' + k]
        err = np.linalg.norm(v - ref) / max(np.linalg.norm(ref), 1e-12)
        assert err < 1e-5, (k, err)


def test_tensorf_realistic_forward_backward(golden):
    """The oracle against LowRankTensor.forward at the benchmark's model shape on
    a 48^3 grid (golden tensorf_realistic: 16 / 48 components, 27 features, 128
    renderer units, a 32^3 alpha mask at 15%, 256 rays, parameters regenerated
    from their seed by oracle.tensorf.seeded_vm_model)."""
    g = golden('tensorf_realistic')
    c = {k[4:]: g[k] for k in g if k.startswith('cfg_')}
    tp, spec = ot.seeded_vm_model(int(c['seed']), [int(c['res'])] * 3, list(c['density']), list(c['color']),
                                  int(c['features']), int(c['units']))
    tp['bbox'] = g['bbox']
    z = ot.aabb_z(g['rays_o'], g['rays_d'], g['bbox'], 2.0, 6.0, float(g['step_size']), int(g['num_samples']), g['u'])
    close(z, g['z'], rtol=1e-6, atol=1e-6)
    out, cache = ot.tensorf_forward(tp, spec, g['rays_o'], g['rays_d'], g['z'], alpha_vol=g['alpha_vol'].astype(np.float32),
                                    alpha_bbox=g['bbox'], white=True)
    assert int((g['out_weights'] > 1e-4).sum()) > 5000
    for k in ('rgb', 'depth', 'acc', 'weights', 'raw_sigma', 'depth_var'):
        ref = g['out_' + k]
        close(out[k], ref, rtol=1e-5, atol=1e-6 * max(1.0, float(np.abs(ref).max())))
    grads = ot.tensorf_backward(tp, spec, cache, {k: g[f'cot_{k}'] for k in ('rgb', 'depth', 'acc')})
    assert len(grads) == 19
    for k, v in grads.items():
        ref = g['grad_' + k]
        err = np.linalg.norm(v - ref) / max(np.linalg.norm(ref), 1e-12)
        assert err < 1e-5, (k, err)


def test_alpha_mask_query(golden):
    g = golden('tensorf')
    pos = ot.grid_sample_3d_positive(g['alpha_vol'], ot.normalize_points(g['alpha_q'], g['bbox']))
    assert np.array_equal(pos, g['alpha_q_pos'])


def test_alpha_mask_rebuild(golden):
    """LowRankTensor.update_alpha_mask (SimpleTensoRF09.py:849-876) restated on the
    oracle's VM density: alpha = 1 - exp(-relu(density) step) on the grid nodes,
    3^3 max-pool, threshold 1e-4, against the reference's volume (golden
    tensorf_maintenance)."""
    import torch
    g = golden('tensorf_maintenance')
    res, bbox = g['res'], g['bbox']
    t = [np.linspace(0, 1, r, dtype=np.float32) for r in res]
    s = np.stack(np.meshgrid(*t, indexing='ij'), -1)
    xyz = bbox[0] * (1 - s) + bbox[1] * s
    pn = ((xyz - bbox[0]) / (bbox[1] - bbox[0]) * 2 - 1).reshape(-1, 3).astype(np.float32)
    planes = [g[f'amask_planes_density.{i}'] for i in range(3)]
    lines = [g[f'amask_lines_density.{i}'] for i in range(3)]
    alpha = 1 - np.exp(-np.maximum(ot.vm_density(planes, lines, pn), 0) * g['amask_step_size'])
    a = torch.from_numpy(alpha.reshape(tuple(res))).transpose(0, 2).contiguous()[None, None]
    a = torch.nn.functional.max_pool3d(a, 3, 1, 1).view(tuple(res[::-1]))
    vol = (a >= 1e-4).float().numpy()
    assert np.array_equal(vol, g['amask_volume'])
    occ = np.argwhere(vol > 0.5)[:, ::-1]   # (x, y, z) node indices of the occupied voxels
    box = bbox[0] + (bbox[1] - bbox[0]) * np.stack([occ.min(0), occ.max(0)]) / (res - 1)
    np.testing.assert_allclose(box, g['amask_box'], rtol=1e-6, atol=1e-6)
