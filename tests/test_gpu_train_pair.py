"""The fused training step in its main + augmented NDC form against the oracle.

Workload: forward-facing NDC rays (H 378, W 504, focal 400, near 1), main coarse
and fine nets, one augmented coarse net (PE L=4 on xyz, no view directions) on
the same coarse samples, loss = MSE of every net's rgb + 0.1 * mean squared
difference of the main coarse depth and the (detached) augmented coarse depth.

FP32 plain path: rgb/acc/depth_ndc/weights within 1e-5 relative of the float32
oracle (acc with an absolute allowance of one ulp(1) per sample), metric depth
within 1e-5 of the reduction of the GPU's weights; parameter gradients of all
three nets within max(1e-4, 3x the float32 oracle's own error) relative L2 per
tensor of the float64 oracle.  BF16 path: rgb within 2e-3 max-abs and whole-gradient relative
L2 per net within 3e-2 of the float64 oracle.  The fine pass is compared on the
depths the GPU sampled.
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


def _run(precision, n_rays=96, seed=5, last_u_max=1.0):
    from simple_rf_gb300.train_step import make_step
    step, batch_fn = make_step('nerf_pair', n_rays, precision, DEV, seed=seed)
    batch = batch_fn(seed + 1, DEV)
    batch[4][:, -1] *= last_u_max
    step.set_batch(*batch)
    params = {tag: {k: v.double().cpu().numpy() for k, v in net.state_dict().items()} for tag, net in step.nets.items()}
    step.step()
    torch.cuda.synchronize()
    out = {k: v.detach().cpu().numpy() for k, v in step.outputs().items()}
    grads = {tag: {k: g.double().cpu().numpy() for k, g in zip(net.spec.param_names, net.gviews)}
             for tag, net in step.nets.items()}
    host = [x.cpu().numpy() for x in batch]
    return step, params, out, grads, host


def _oracle(params, host, z_fine, dtype):
    o, d, t_rgb, _, u_c, u_f = [np.asarray(x, dtype) for x in host]
    n = o.shape[0]
    spec = on.MlpSpec()
    aspec = on.MlpSpec(points_pe_degree=4, use_view_dirs=False, view_dependent_rgb=False)
    p = {tag: {k: v.astype(dtype) for k, v in params[tag].items()} for tag in params}
    focal = np.full(n, 400.0, dtype)
    ndc = dict(h=378, w=504, fx=focal, fy=focal, near=1.0)
    aug = [(AUG, {'coarse': p[f'{AUG}_coarse']}, aspec)]
    ret, caches = on.render_rays(p['coarse'], p['fine'], spec, spec, o, d, 0.0, 1.0, 64, 128, u_c, u_f,
                                 ndc=ndc, aug=aug, z_fine=z_fine.astype(dtype), pts_fp32=True)
    g = {}
    dt = dtype
    for tag, key in (('coarse', 'rgb_coarse'), ('fine', 'rgb_fine'), (f'{AUG}_coarse', f'{AUG}_rgb_coarse')):
        g[f'rgb_{tag}'] = (dt(2.0) / dt(3 * n)) * (ret[key] - t_rgb)
    e = ret['depth_coarse'] - ret[f'{AUG}_depth_coarse']
    g['depth_coarse'] = dt(2 * 0.1) * e / dt(n)
    specs = {'coarse': spec, 'fine': spec, f'{AUG}_coarse': aspec}
    grads = on.backward_render(p, specs, caches, g, n)
    return ret, grads


def _ret_key(k, tag):
    key = {'rgb_map': 'rgb'}.get(k, k)
    if tag.startswith(AUG):
        return f'{AUG}_{key}_coarse'
    return f'{key}_{tag}'


def test_fp32_pair_step_matches_oracle():
    """Outputs of the FP32 plain pair step vs the float32 oracle.

    The metric depth of an NDC ray is sum_i w_i m(z_i) / (acc + 1e-6) with
    m(z) affine in 1 / (1 - z) (SimpleNeRF17.py:526-558) and the last jittered sample has 1 - z_i down to
    ~1e-7, so a float32 rounding of a 1e-8 weight moves the depth by 1e-3: it is
    checked as the reduction of the GPU's own weights (in float64), while the
    well-conditioned outputs (rgb, acc, weights, NDC depth) are compared with the
    oracle directly."""
    step, params, out, grads, host = _run('fp32')
    assert set(step.nets) == {'coarse', 'fine', f'{AUG}_coarse'}
    ret32, _ = _oracle(params, host, out['z_fine'], np.float32)
    np.testing.assert_allclose(out['z_coarse'], ret32['z_vals_coarse'], rtol=0, atol=1e-7)
    o64, d64 = np.asarray(host[0], np.float64), np.asarray(host[1], np.float64)
    for tag in ('coarse', 'fine', f'{AUG}_coarse'):
        for k in ('rgb_map', 'depth_ndc', 'weights', 'acc'):
            ref = ret32[_ret_key(k, tag)]
            # acc sums one alpha = 1 - exp(-sigma delta) per sample, each carrying an
            # absolute rounding of up to ulp(1) = 2^-23 from the subtraction
            atol = out[f'weights_{tag}'].shape[1] * 2.0 ** -23 if k == 'acc' else \
                1e-6 * max(1.0, float(np.abs(ref).max()))
            np.testing.assert_allclose(out[f'{k}_{tag}'], ref, rtol=1e-5, atol=atol, err_msg=f'{k}_{tag}')
        w = out[f'weights_{tag}'].astype(np.float64)
        zm = on.depth_from_ndc(out[f'z_{tag}'].astype(np.float64), o64, d64)
        ref = np.sum(w * zm, -1) / (np.sum(w, -1) + 1e-6)
        np.testing.assert_allclose(out[f'depth_{tag}'], ref, rtol=1e-5, atol=1e-6 * float(np.abs(ref).max()),
                                   err_msg=f'depth_{tag}')


def test_fp32_pair_step_gradients_against_fp64_oracle():
    """Parameter gradients of all three nets vs the float64 oracle.  The last
    coarse uniform is drawn from [0, 0.5) so 1 - z_last >= (1 - z_mid) / 2 and the
    metric depth feeding the consistency term stays well conditioned."""
    from test_gpu_train_step import check_fp32_gradients
    step, params, out, grads, host = _run('fp32', last_u_max=0.5)
    _, g64 = _oracle(params, host, out['z_fine'], np.float64)
    _, g32 = _oracle(params, host, out['z_fine'], np.float32)
    assert set(g64) == set(step.nets)
    check_fp32_gradients(grads, g32, g64)


def test_consistency_term_reaches_main_coarse_only():
    """With the consistency weight at 0 the main coarse gradient changes and the
    others do not (the augmented depth is a detached target)."""
    from simple_rf_gb300.train_step import make_step
    res = {}
    for w in (0.1, 0.0):
        step, batch_fn = make_step('nerf_pair', 64, 'fp32', DEV, seed=2, consistency_weight=w)
        step.set_batch(*batch_fn(3, DEV))
        step.step()
        torch.cuda.synchronize()
        res[w] = {tag: net.grad.clone() for tag, net in step.nets.items()}

    def close(a, b):
        # the FP32 weight gradients sum with atomics: equal up to summation order
        return torch.allclose(a, b, rtol=1e-5, atol=1e-6 * float(b.abs().max()))

    assert not close(res[0.1]['coarse'], res[0.0]['coarse'])
    assert close(res[0.1]['fine'], res[0.0]['fine'])
    assert close(res[0.1][f'{AUG}_coarse'], res[0.0][f'{AUG}_coarse'])


def test_bf16_pair_step_against_fp64_oracle():
    step, params, out, grads, host = _run('bf16')
    ret64, g64 = _oracle(params, host, out['z_fine'], np.float64)
    for tag in ('coarse', 'fine', f'{AUG}_coarse'):
        err = np.abs(out[f'rgb_map_{tag}'] - ret64[_ret_key('rgb_map', tag)]).max()
        assert err < 2e-3, (tag, err)
        got = np.concatenate([grads[tag][k].ravel() for k in g64[tag]])
        ref = np.concatenate([g64[tag][k].ravel() for k in g64[tag]])
        rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        print(tag, 'whole-gradient rel-L2', rel)
        assert rel < 3e-2, (tag, rel)


def test_pair_graph_replay_equals_eager():
    from simple_rf_gb300.train_step import make_step
    a, batch_fn = make_step('nerf_pair', 256, 'bf16', DEV, seed=1)
    b, _ = make_step('nerf_pair', 256, 'bf16', DEV, seed=1)
    batch = batch_fn(4, DEV)
    a.set_batch(*batch)
    a.step()
    b.set_batch(*batch)
    b.capture(warmup=0)
    b.step()
    torch.cuda.synchronize()
    for tag in a.buf:
        for k in ('rgb_map', 'depth', 'z'):
            assert torch.equal(a.buf[tag][k], b.buf[tag][k]), (k, tag)
