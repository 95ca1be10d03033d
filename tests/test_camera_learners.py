"""Learnt camera parameters of the drop-in models against the reference's own
classes (golden camera_learners.npz from ExtrinsicsLearner and IntrinsicsLearner,
SimpleNeRF17.py:788-912): the extrinsics composed from seeded axis-angle and
translation deltas (one frame with a zero rotation), repeated frame ids, and the
gradients that flow back into the deltas.  Host-side PyTorch on the CPU: the
camera learners launch no kernel of the library."""
import os

import numpy as np
import torch

from simple_rf_gb300.nerf import ExtrinsicsLearner, IntrinsicsLearner

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden', 'camera_learners.npz')


def test_extrinsics_and_gradients_match_reference():
    g = np.load(GOLDEN)
    el = ExtrinsicsLearner(g['init_extrinsics'], learn_rotation=True, learn_translation=True)
    with torch.no_grad():
        el.r.copy_(torch.from_numpy(g['r']))
        el.t.copy_(torch.from_numpy(g['t']))
    ext = el(torch.from_numpy(g['ids']))
    (ext * torch.from_numpy(g['wsum'])).sum().backward()
    # fp32 Rodrigues rotation and a 4x4 inverse on both sides
    np.testing.assert_allclose(ext.detach().numpy(), g['extrinsics'], rtol=0, atol=1e-5)
    np.testing.assert_allclose(el.r.grad.numpy(), g['grad_r'], rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(el.t.grad.numpy(), g['grad_t'], rtol=1e-4, atol=1e-4)


def test_intrinsics_lookup_and_frozen_flags():
    g = np.load(GOLDEN)
    il = IntrinsicsLearner(g['init_intrinsics'], learn_focal=False)
    np.testing.assert_array_equal(il(torch.from_numpy(g['ids'])).numpy(), g['intrinsics'])
    assert not il.initial_intrinsics.requires_grad
    el = ExtrinsicsLearner(g['init_extrinsics'], learn_rotation=False, learn_translation=True)
    assert not el.r.requires_grad and el.t.requires_grad and not el.initial_extrinsics.requires_grad
    # zero deltas leave the initial poses unchanged
    ext = el(torch.arange(len(g['init_extrinsics'])))
    np.testing.assert_allclose(ext.detach().numpy(), g['init_extrinsics'], rtol=0, atol=1e-6)
    groups = el.get_trainable_parameters({'lr_initial': 1e-3})
    assert [gr['name'] for gr in groups] == ['ExtrinsicsLearner_params'] and groups[0]['lr'] == 1e-3


def test_pose_learning_is_refused_in_training_and_allowed_in_evaluation():
    """With learn_camera_rotation / learn_camera_translation on, a training pass of
    the drop-in raises NotImplementedError (the rays carry no gradient to the
    extrinsics) before any work; evaluation mode passes the check."""
    import pytest
    import torch
    from simple_rf_gb300.nerf import GbSimpleNeRF, check_pose_learning
    mc = {'num_samples': 8, 'points_net_depth': 8, 'views_net_depth': 1, 'points_net_width': 256,
          'views_net_width': 128, 'points_positional_encoding_degree': 10, 'views_positional_encoding_degree': 4,
          'use_view_dirs': True, 'view_dependent_rgb': True, 'predict_visibility': False}
    for rot, trans in ((True, False), (False, True)):
        configs = {'data_loader': {'ndc': False}, 'model': {
            'name': 'GbSimpleNeRF01', 'coarse_model': mc, 'learn_camera_focal_length': False,
            'learn_camera_rotation': rot, 'learn_camera_translation': trans, 'chunk': 64, 'lindisp': False,
            'netchunk': 64, 'perturb': False, 'raw_noise_std': 0.0, 'white_bkgd': False}}
        model = GbSimpleNeRF(configs, {'intrinsics': np.eye(3)[None], 'extrinsics': np.eye(4)[None],
                                       'resolution': (8, 8), 'near': 2.0, 'far': 6.0})
        model.train()
        with pytest.raises(NotImplementedError):
            model({'pixel_id': torch.zeros(4, 3, dtype=torch.int32), 'num_frames': 1})
        model.eval()
        check_pose_learning(model)
