"""Recomputation mode of the NeRF MLP op: with an activation budget below what
the backward would keep, the forward stores nothing and the backward recomputes
each ray chunk's activations before its adjoint.

Bars: sigma/rgb bit-identical to the stored-activation pass in FP32 (same
kernels on the same rows) and within 1e-6 relative with 16-bit operands (the
forward that stores nothing runs the fused MLP kernel, whose head dot products
sum their partials in another order than the per-layer kernels); parameter
gradients within 1e-5 (FP32) / 1e-4 (16-bit operands) relative L2 of the
stored-activation pass -- only the grouping of the sum over samples differs."""
import numpy as np
import pytest
import torch

from oracle import nerf as on

pytestmark = pytest.mark.gpu
DEV = 'cuda'


@pytest.fixture(scope='module', autouse=True)
def built():
    from simple_rf_gb300 import build as b
    b.build()


def _run(spec, prec, pts, vd, div, p64, cs, cr, budget):
    from simple_rf_gb300 import functional as F
    params = [torch.from_numpy(p64[k].astype(np.float32)).to(DEV).requires_grad_(True) for k in spec.param_names]
    with F.activation_budget(budget):
        sigma, rgb = F.NerfMlpFunction.apply(spec, prec, pts, vd, div, None, *params)
    ((sigma * cs).sum() + (rgb * cr).sum()).backward()
    torch.cuda.synchronize()
    return sigma.detach(), rgb.detach(), [p.grad.double() for p in params]


@pytest.mark.parametrize('precision', ['fp32', 'bf16', 'fp16'])
def test_recomputed_backward_matches_stored_activations(precision):
    from simple_rf_gb300 import _lib
    from simple_rf_gb300 import functional as F
    spec = F.MlpSpec()
    prec = _lib.PRECISIONS[precision]
    p64 = on.xavier_params(on.MlpSpec(), 31, np.float64)
    rng = np.random.default_rng(32)
    div, n_rays = 192, 64
    m = div * n_rays
    pts = torch.from_numpy((rng.standard_normal((m, 3)) * 0.7).astype(np.float32)).to(DEV)
    vd = rng.standard_normal((n_rays, 3))
    vd = torch.from_numpy((vd / np.linalg.norm(vd, axis=1, keepdims=True)).astype(np.float32)).to(DEV)
    cs = torch.from_numpy(rng.standard_normal(m).astype(np.float32)).to(DEV)
    cr = torch.from_numpy(rng.standard_normal((m, 3)).astype(np.float32)).to(DEV)
    full = spec.workspace_bytes(m, prec, True)
    budget = spec.workspace_bytes(3 * 384, prec, True)
    rows = F.recompute_rows(m, div, budget, lambda r: spec.workspace_bytes(r, prec, True))
    assert rows == 3 * 384 and m % rows != 0  # 11 chunks, the last one partial
    s0, r0, g0 = _run(spec, prec, pts, vd, div, p64, cs, cr, 2 * full)
    s1, r1, g1 = _run(spec, prec, pts, vd, div, p64, cs, cr, budget)
    if precision == 'fp32':
        assert torch.equal(s0, s1) and torch.equal(r0, r1)
    else:
        torch.testing.assert_close(s1, s0, rtol=1e-6, atol=1e-6 * max(1.0, float(s0.abs().max())))
        torch.testing.assert_close(r1, r0, rtol=1e-6, atol=1e-6)
    bar = 1e-5 if precision == 'fp32' else 1e-4
    for name, a, b in zip(spec.param_names, g0, g1):
        rel = float(torch.linalg.norm(a - b) / torch.linalg.norm(a).clamp_min(1e-30))
        assert rel < bar, (name, rel)


def test_drop_in_model_activation_budget_config():
    """configs['model']['activation_budget_bytes'] on the drop-in GbSimpleNeRF:
    the same rendered outputs and (within 1e-5 relative L2) the same parameter
    gradients as without a budget, with the backward recomputing ray chunks."""
    from simple_rf_gb300.nerf import GbSimpleNeRF
    mc = {'num_samples': 64, 'points_net_depth': 8, 'views_net_depth': 1, 'points_net_width': 256,
          'views_net_width': 128, 'points_positional_encoding_degree': 10, 'views_positional_encoding_degree': 4,
          'use_view_dirs': True, 'view_dependent_rgb': True, 'predict_visibility': False}
    mf = dict(mc, num_samples=128)
    intr = np.array([[300.0, 0, 32.0], [0, 300.0, 32.0], [0, 0, 1.0]])
    ext = np.eye(4)
    model_configs = {'intrinsics': intr[None], 'extrinsics': ext[None], 'resolution': (64, 64), 'near': 2.0,
                     'far': 6.0, 'near_ndc': 0.0, 'far_ndc': 1.0}
    rng = np.random.default_rng(3)
    pix = np.stack([np.zeros(256), rng.integers(0, 64, 256), rng.integers(0, 64, 256)], 1).astype(np.int32)
    grads, outs = [], []
    for budget in (None, 8 << 20):
        model_cfg = {'name': 'GbSimpleNeRF01', 'coarse_model': mc, 'fine_model': mf, 'learn_camera_focal_length': False,
                     'learn_camera_rotation': False, 'learn_camera_translation': False, 'chunk': 4096,
                     'lindisp': False, 'netchunk': 16384, 'perturb': False, 'raw_noise_std': 0.0, 'white_bkgd': True}
        if budget is not None:
            model_cfg['activation_budget_bytes'] = budget
        torch.manual_seed(0)
        model = GbSimpleNeRF({'data_loader': {'ndc': False}, 'model': model_cfg}, model_configs).to(DEV)
        spec = on.MlpSpec()
        with torch.no_grad():
            for mod, seed in ((model.coarse_model, 0), (model.fine_model, 1)):
                p = on.xavier_params(spec, seed)
                for name, prm in mod.named_parameters():
                    prm.copy_(torch.from_numpy(p[name]))
        batch = {'pixel_id': torch.from_numpy(pix).to(DEV), 'num_frames': 1, 'common_data': {}}
        ret = model(batch, retraw=True)
        (ret['rgb_coarse'].sum() + ret['rgb_fine'].sum() + 0.1 * ret['depth_fine'].sum()).backward()
        outs.append(ret['rgb_fine'].detach())
        grads.append([p.grad.detach().double().clone() for p in list(model.coarse_model.parameters()) +
                      list(model.fine_model.parameters())])
    assert torch.equal(outs[0], outs[1])
    for a, b in zip(*grads):
        assert float(torch.linalg.norm(a - b) / torch.linalg.norm(a).clamp_min(1e-30)) < 1e-5
