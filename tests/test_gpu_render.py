"""Chunked full-image render of the main + augmented NeRF pair against the oracle.

Two 24x20 forward-facing views (960 rays) in chunks of 256, so the last chunk is
partial (192 rays on a padded batch).  FP32 plain path: coarse, fine and augmented
rgb/acc within 1e-5 relative of the float32 oracle (acc with an absolute allowance
of one ulp(1) per sample) (deterministic samples, no
jitter; the fine pass is compared on the depths the GPU sampled).  The BF16 graph
render equals the BF16 eager render bit for bit.
"""
import numpy as np
import pytest
import torch

from oracle import nerf as on

pytestmark = pytest.mark.gpu
DEV = 'cuda'
AUG = 'views_augmentation'


@pytest.fixture(scope='module', autouse=True)
def built():
    from simple_rf_gb300 import build as b
    b.build()


def _rays():
    from simple_rf_gb300.render import pixel_rays, synthetic_views
    pid, intr, ext = synthetic_views(2, 20, 24, focal=30.0, seed=3, device=DEV)
    return pixel_rays(pid, intr, ext)


def test_fp32_render_matches_oracle():
    from simple_rf_gb300.render import NerfPairRenderer
    o, d = _rays()
    r = NerfPairRenderer(256, 'fp32', DEV, seed=4, graph=False)
    out = r.render(o, d, keep=('rgb', 'acc', 'z'))
    torch.cuda.synchronize()
    params = {tag: {k: v.cpu().numpy() for k, v in net.state_dict().items()} for tag, net in r.nets.items()}
    on_o, on_d = o.cpu().numpy(), d.cpu().numpy()
    n = on_o.shape[0]
    spec = on.MlpSpec()
    aspec = on.MlpSpec(points_pe_degree=4, use_view_dirs=False, view_dependent_rgb=False)
    focal = np.full(n, 400.0, np.float32)
    ret, _ = on.render_rays(params['coarse'], params['fine'], spec, spec, on_o, on_d, 0.0, 1.0, 64, 128,
                            ndc=dict(h=378, w=504, fx=focal, fy=focal, near=1.0),
                            aug=[(AUG, {'coarse': params[f'{AUG}_coarse']}, aspec)],
                            z_fine=out['fine']['z'].cpu().numpy())
    # torch.linspace rounds host-dependently: the midpoint depths agree within an ulp
    np.testing.assert_allclose(out['coarse']['z'].cpu().numpy(), ret['z_vals_coarse'], rtol=0, atol=1.2e-7)
    for tag, pre in (('coarse', ''), ('fine', ''), (f'{AUG}_coarse', f'{AUG}_')):
        lvl = 'fine' if tag == 'fine' else 'coarse'
        n_s = out[tag]['z'].shape[1]
        for k in ('rgb', 'acc'):
            ref = ret[f'{pre}{k}_{lvl}']
            # acc sums one alpha = 1 - exp(-sigma delta) per sample, each with an
            # absolute rounding of up to ulp(1) = 2^-23 from the subtraction
            atol = n_s * 2.0 ** -23 if k == 'acc' else 1e-6
            np.testing.assert_allclose(out[tag][k].cpu().numpy(), ref, rtol=1e-5, atol=atol, err_msg=f'{k}_{tag}')


def test_bf16_graph_render_equals_eager():
    from simple_rf_gb300.render import NerfPairRenderer
    o, d = _rays()
    a = NerfPairRenderer(256, 'bf16', DEV, seed=4, graph=False).render(o, d)
    b = NerfPairRenderer(256, 'bf16', DEV, seed=4, graph=True).render(o, d)
    torch.cuda.synchronize()
    for tag in a:
        for k in a[tag]:
            assert torch.equal(a[tag][k], b[tag][k]), (tag, k)


def test_drop_in_output_dicts_match_reference_keys(golden):
    """The drop-in models' forward output dicts carry the reference's keys with
    the reference's shapes (golden output_keys from SimpleNeRF / SimpleTensoRF on
    8 pixels of one frame), in training mode (augmented models, raw outputs) and
    in evaluation mode: the contract Trainer10, Tester07 and the losses read."""
    from simple_rf_gb300.nerf import GbSimpleNeRF
    from simple_rf_gb300.tensorf_model import GbSimpleTensoRF
    g = golden('output_keys')

    def mlp(ns, lp=10, lv=4, views=True, vdr=True, lps=None):
        c = {'num_samples': ns, 'points_net_depth': 8, 'views_net_depth': 1, 'points_net_width': 256,
             'views_net_width': 128, 'points_positional_encoding_degree': lp, 'views_positional_encoding_degree': lv,
             'use_view_dirs': views, 'view_dependent_rgb': vdr, 'predict_visibility': False}
        if lps is not None:
            c['points_sigma_positional_encoding_degree'] = lps
        return c

    def tcfg(vox):
        return {'decomposition_type': 'VectorMatrix', 'num_samples_max': 1e6, 'num_components_density': [16, 4, 4],
                'num_components_color': [48, 12, 12], 'bounding_box': [[-1.5, -1.67, -1.0], [1.5, 1.67, 1.0]],
                'num_voxels_initial': vox, 'num_voxels_final': vox, 'tensor_upsampling_iters': [],
                'num_voxels_per_sample': 0.5, 'alpha_mask_update_iters': [], 'alpha_mask_threshold': 1e-4,
                'ray_marching_weight_threshold': 1e-4, 'use_view_dirs': True, 'view_dependent_color': True,
                'views_positional_encoding_degree': 0, 'features_positional_encoding_degree': 0,
                'features_dimension_color': 27, 'density_offset': -10, 'distance_scale': 25,
                'density_predictor': 'ReLU', 'color_predictor': 'MLP_Features', 'num_units_color_predictor': 128,
                'predict_visibility': False}

    mc = {'intrinsics': np.array([[[400.0, 0, 252.0], [0, 400.0, 189.0], [0, 0, 1.0]]]), 'extrinsics': np.eye(4)[None],
          'resolution': (378, 504), 'near': 1.0, 'far': 6.0, 'near_ndc': 0.0, 'far_ndc': 1.0}
    cams = {'learn_camera_focal_length': False, 'learn_camera_rotation': False, 'learn_camera_translation': False}
    nerf = GbSimpleNeRF({'data_loader': {'ndc': True}, 'database': 'synthetic', 'model': dict(
        cams, name='GbSimpleNeRF01', coarse_model=mlp(16), fine_model=mlp(32), chunk=1 << 20, lindisp=False,
        netchunk=1 << 20, perturb=True, raw_noise_std=0.0, white_bkgd=False,
        augmentations=[{'name': 'views_augmentation', 'coarse_model': mlp(16, lp=4, views=False, vdr=False)},
                       {'name': 'points_augmentation', 'coarse_model': mlp(16, lps=3)}])}, mc)
    bbox = np.array([[-1.5, -1.67, -1.0], [1.5, 1.67, 1.0]])
    tensorf = GbSimpleTensoRF({'data_loader': {'ndc': True}, 'database': 'NeRF_LLFF', 'model': dict(
        cams, name='GbSimpleTensoRF01', coarse_model=tcfg(24 ** 3), chunk=1 << 16, lindisp=False, perturb=True,
        white_bkgd=False, augmentations=[{'name': 'points_augmentation', 'coarse_model': tcfg(12 ** 3)}])},
        dict(mc, bounding_box=bbox))
    batch = {'pixel_id': torch.from_numpy(g['pixel_id']).to(DEV), 'num_frames': 1, 'iter_num': 1,
             'sub_batch_index': 1, 'common_data': {}}
    for tag, m in (('nerf', nerf.to(DEV)), ('tensorf', tensorf.to(DEV))):
        for mode, train in (('train', True), ('eval', False)):
            m.train(train)
            with torch.set_grad_enabled(train):
                ret = m(batch, retraw=False)
            got = sorted(f"{k}:{'x'.join(str(d) for d in v.shape)}" for k, v in ret.items()
                         if isinstance(v, torch.Tensor))
            assert got == list(g[f'{tag}_{mode}']), (tag, mode, sorted(set(got) ^ set(g[f'{tag}_{mode}'])))
