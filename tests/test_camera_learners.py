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
