"""The drop-in models keep the reference's state_dict and optimizer parameter
groups: the same keys in the same order with the same shapes, and the same
groups (names, learning rates, parameter shapes in order), as the reference's
SimpleNeRF and SimpleTensoRF built from the same configurations (golden
state_dicts.npz from the reference's own classes), so checkpoints written by
either load into the other (Trainer10.py:364-394) and the optimizer state lines
up (Trainer10.py:509-520).  Built on the CPU: construction launches no kernel."""
import numpy as np
import pytest

TBOX = [[-1.5, -1.67, -1.0], [1.5, 1.67, 1.0]]


def _mlp(ns=64, lp=10, lv=4, views=True, vdr=True, lps=None):
    c = {'num_samples': ns, 'points_net_depth': 8, 'views_net_depth': 1, 'points_net_width': 256,
         'views_net_width': 128, 'points_positional_encoding_degree': lp, 'views_positional_encoding_degree': lv,
         'use_view_dirs': views, 'view_dependent_rgb': vdr, 'predict_visibility': False}
    if lps is not None:
        c['points_sigma_positional_encoding_degree'] = lps
    return c


def _model_configs():
    return {'intrinsics': np.eye(3)[None], 'extrinsics': np.eye(4)[None], 'resolution': (378, 504), 'near': 1.0,
            'far': 6.0, 'near_ndc': 0.0, 'far_ndc': 1.0}


def _tcfg(vox):
    return {'decomposition_type': 'VectorMatrix', 'num_samples_max': 1e6, 'num_components_density': [16, 4, 4],
            'num_components_color': [48, 12, 12], 'bounding_box': TBOX, 'num_voxels_initial': vox,
            'num_voxels_final': vox, 'tensor_upsampling_iters': [], 'num_voxels_per_sample': 0.5,
            'alpha_mask_update_iters': [], 'alpha_mask_threshold': 1e-4, 'ray_marching_weight_threshold': 1e-4,
            'use_view_dirs': True, 'view_dependent_color': True, 'views_positional_encoding_degree': 0,
            'features_positional_encoding_degree': 0, 'features_dimension_color': 27, 'density_offset': -10,
            'distance_scale': 25, 'density_predictor': 'ReLU', 'color_predictor': 'MLP_Features',
            'num_units_color_predictor': 128, 'predict_visibility': False}


def _signature(model):
    return [f"{k}:{'x'.join(str(d) for d in v.shape)}" for k, v in model.state_dict().items()]


OPT = {'lr_initial': 5e-4, 'lr_initial_tensor': 0.02, 'lr_initial_network': 1e-3}


def _groups(model):
    """The optimizer's parameter groups as the trainer builds them (Trainer10.py:509-520)."""
    return [f"{g['name']}|{g['lr']}|" + ','.join('x'.join(str(d) for d in p.shape) for p in g['params'])
            for g in model.get_trainable_parameters(OPT)]


def test_nerf_state_dict_matches_reference(golden):
    pytest.importorskip('torch')
    from simple_rf_gb300.nerf import GbSimpleNeRF
    augs = [{'name': 'views_augmentation', 'coarse_model': _mlp(lp=4, views=False, vdr=False)},
            {'name': 'points_augmentation', 'coarse_model': _mlp(lps=3)}]
    model = {'name': 'GbSimpleNeRF01', 'coarse_model': _mlp(), 'fine_model': _mlp(ns=128),
             'learn_camera_focal_length': False, 'learn_camera_rotation': False, 'learn_camera_translation': False,
             'chunk': 1 << 20, 'lindisp': False, 'netchunk': 1 << 20, 'perturb': True, 'raw_noise_std': 0.0,
             'white_bkgd': False, 'augmentations': augs}
    m = GbSimpleNeRF({'data_loader': {'ndc': True}, 'model': model, 'database': 'synthetic'}, _model_configs())
    assert _signature(m) == list(golden('state_dicts')['nerf_keys'])
    assert _groups(m) == list(golden('state_dicts')['nerf_groups'])


def test_tensorf_state_dict_matches_reference(golden):
    pytest.importorskip('torch')
    from simple_rf_gb300.tensorf_model import GbSimpleTensoRF
    model = {'name': 'GbSimpleTensoRF01', 'coarse_model': _tcfg(24 ** 3),
             'augmentations': [{'name': 'points_augmentation', 'coarse_model': _tcfg(12 ** 3)}],
             'learn_camera_focal_length': False, 'learn_camera_rotation': False, 'learn_camera_translation': False,
             'chunk': 1 << 16, 'lindisp': False, 'perturb': True, 'white_bkgd': False}
    mc = dict(_model_configs(), bounding_box=np.array(TBOX))
    m = GbSimpleTensoRF({'data_loader': {'ndc': True}, 'model': model, 'database': 'NeRF_LLFF'}, mc)
    assert _signature(m) == list(golden('state_dicts')['tensorf_keys'])
    assert _groups(m) == list(golden('state_dicts')['tensorf_groups'])


def test_tensorf_checkpoint_of_another_resolution_loads():
    """A checkpoint written after the grid was upsampled (and an alpha mask built)
    loads into a model constructed at the initial resolution: the load hook
    (SimpleTensoRF09.py:946-961, 1196-1212) rebuilds the alpha mask and resizes
    the planes and lines first, and every tensor then equals the checkpoint's."""
    torch = pytest.importorskip('torch')
    from simple_rf_gb300.tensorf_model import AlphaGridMask, GbSimpleTensoRF

    def build(vox):
        model = {'name': 'GbSimpleTensoRF01', 'coarse_model': _tcfg(vox), 'learn_camera_focal_length': False,
                 'learn_camera_rotation': False, 'learn_camera_translation': False, 'chunk': 1 << 16,
                 'lindisp': False, 'perturb': True, 'white_bkgd': False}
        mc = dict(_model_configs(), bounding_box=np.array(TBOX))
        return GbSimpleTensoRF({'data_loader': {'ndc': True}, 'model': model, 'database': 'NeRF_LLFF'}, mc)

    src, dst = build(24 ** 3), build(12 ** 3)
    vol = torch.rand(10, 12, 14, generator=torch.Generator().manual_seed(0)) < 0.3
    src.coarse_model.alpha_mask = AlphaGridMask(vol, torch.tensor(TBOX))
    sd = src.state_dict()
    assert sd['coarse_model.alpha_mask.alpha_volume'].dtype == torch.bool
    dst.load_state_dict(sd)
    out = dst.state_dict()
    assert list(out) == list(sd)
    for k, v in sd.items():
        assert out[k].shape == v.shape and torch.equal(out[k].to(v.dtype), v), k


def _vm_from_golden(g):
    torch = pytest.importorskip('torch')
    from simple_rf_gb300 import tensorf as T
    from simple_rf_gb300.tensorf_model import GbVmTensor
    bbox = g['bbox'].tolist()
    tcfg = dict(_tcfg(int(np.prod(g['res']))), bounding_box=bbox, num_components_density=[4, 3, 2],
                num_components_color=[6, 5, 4], views_positional_encoding_degree=2,
                features_positional_encoding_degree=2, features_dimension_color=7, num_units_color_predictor=16)
    tm = GbVmTensor('coarse_model', {'data_loader': {'ndc': False}, 'model': {'white_bkgd': False}}, tcfg,
                    {'bounding_box': bbox})
    tm.update_tensor_params(torch.tensor(g['res']), torch.tensor(g['bbox']))
    with torch.no_grad():
        for kind, plist in (('planes_density', tm.matrices_density), ('lines_density', tm.vectors_density),
                            ('planes_color', tm.matrices_color), ('lines_color', tm.vectors_color)):
            for i in range(3):
                plist[i] = torch.nn.Parameter(T.to_channels_last(torch.from_numpy(g[f'{kind}.{i}'])[None]))
    return tm


def _grids(tm):
    return {f'{kind}.{i}': plist[i].detach()[0].cpu().numpy()
            for kind, plist in (('planes_density', tm.matrices_density), ('lines_density', tm.vectors_density),
                                ('planes_color', tm.matrices_color), ('lines_color', tm.vectors_color))
            for i in range(3)}


@pytest.mark.gpu
def test_tensorf_grid_upsample_and_shrink_match_reference(golden):
    """The drop-in's grid maintenance kernels (srf_resample_grid, srf_crop_grid) on
    the channels-last tensors against the reference's VmDecomposedTensor (golden
    tensorf_maintenance): bilinear upsampling to a new resolution
    (SimpleTensoRF09.py:1284-1301) within 1e-6, and shrinking to an occupied box
    with an alpha mask of another resolution (:899-914, 1303-1320) exactly, with
    the same resolution, box and sample count."""
    torch = pytest.importorskip('torch')
    from simple_rf_gb300 import build as b
    b.build()
    from simple_rf_gb300.tensorf_model import AlphaGridMask
    g = golden('tensorf_maintenance')
    tm = _vm_from_golden(g).to('cuda')
    tm.resample_tensor(torch.tensor(g['res_up']))
    for k, v in _grids(tm).items():
        np.testing.assert_allclose(v, g[f'up_{k}'], rtol=1e-6, atol=1e-6, err_msg=k)
    tm = _vm_from_golden(g).to('cuda')
    tm.alpha_mask = AlphaGridMask(torch.from_numpy(g['alpha_vol']).cuda(), torch.from_numpy(g['bbox']).cuda())
    tm.shrink_tensor(torch.from_numpy(g['box_new']).cuda())
    for k, v in _grids(tm).items():
        np.testing.assert_array_equal(v, g[f'shrunk_{k}'], err_msg=k)
    np.testing.assert_array_equal(tm.resolution.cpu().numpy(), g['shrunk_res'])
    np.testing.assert_allclose(tm.bounding_box.cpu().numpy(), g['shrunk_bbox'], rtol=1e-6)
    assert int(tm.num_samples) == int(g['shrunk_num_samples'])
    np.testing.assert_allclose(float(tm.step_size), float(g['shrunk_step_size']), rtol=1e-6)


def test_tensorf_cp_state_dict_matches_reference(golden):
    """The CP decomposition (CpDecomposedTensor, SimpleTensoRF09.py:964-1123) as
    the drop-in builds it through the same factory: state_dict and parameter groups."""
    pytest.importorskip('torch')
    from simple_rf_gb300.tensorf_model import GbCpTensor, GbSimpleTensoRF
    cp = dict(_tcfg(24 ** 3), decomposition_type='CandecompParafac', num_components_density=[16],
              num_components_color=[48])
    model = {'name': 'GbSimpleTensoRF01', 'coarse_model': cp, 'learn_camera_focal_length': False,
             'learn_camera_rotation': False, 'learn_camera_translation': False, 'chunk': 1 << 16,
             'lindisp': False, 'perturb': True, 'white_bkgd': False}
    mc = dict(_model_configs(), bounding_box=np.array(TBOX))
    m = GbSimpleTensoRF({'data_loader': {'ndc': True}, 'model': model, 'database': 'NeRF_LLFF'}, mc)
    assert isinstance(m.coarse_model, GbCpTensor)
    assert _signature(m) == list(golden('state_dicts')['tensorf_cp_keys'])
    assert _groups(m) == list(golden('state_dicts')['tensorf_cp_groups'])
