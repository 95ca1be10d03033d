"""The FP32 plain path against the oracle at the full sizes of the benchmark
workloads (the kernel-level tests cover small and ragged shapes):

* NeRF render, 1024 rays, 64 stratified + 128 inverse-CDF samples, separate
  Xavier-initialised coarse and fine 8x256 nets, explicit uniforms from seed 0,
  through the functional path and through the drop-in GbSimpleNeRF;
* NeRF training step, 4096 rays (white background, rgb MSE + 0.1 L1 depth on a
  quarter of the rays): every output of the fused step and the parameter
  gradients of both nets;
* TensoRF VM model, 300^3 grid, 16 / 48 components, 27 features, 128-unit
  renderer, 128^3 alpha mask at 15% occupancy, 8192 rays: outputs of all rays
  and the gradients of every grid and renderer parameter;
* the NDC main + augmented pair step, 4096 rays (FP32 plain against float32,
  the FP16 step's rgb against float64), and one full 504 x 378 view rendered in
  chunks of 65,536 rays.

Tolerances: rgb/depth/weights/acc within 1e-5 relative (absolute floor 1e-6 of
the value range) of the float32 oracle; gradients as in test_gpu_train_step.py
(per tensor within max(1e-4, 3x the float32 oracle's own error) of the float64
oracle) for NeRF, 1e-4 relative L2 against the float32 oracle for TensoRF.

Two places where two correct float32 implementations legitimately disagree are
excluded explicitly, counted, and the count is asserted to be tiny:

* NeRF, the last sample of a world-space ray (delta = 1e10 |d|,
  SimpleNeRF17.py:489-492): when its raw sigma pre-activation lies within
  rounding of 0, one side has sigma = 0 and the other alpha = 1.  Rays whose
  last sigma is zero on one side only are dropped from the output comparison.
* TensoRF, the surface threshold (weights > 1e-4, SimpleTensoRF09.py:726): a
  sample whose weight lies within float32 rounding of 1e-4 may be coloured on
  one side only.  Rays with a sample whose two weights straddle the threshold,
  or lie within 1e-5 relative of it, are dropped from the comparison.
"""
import numpy as np
import pytest
import torch

from oracle import nerf as on
from oracle import tensorf as ot

pytestmark = pytest.mark.gpu
DEV = 'cuda'


@pytest.fixture(scope='module', autouse=True)
def built():
    from simple_rf_gb300 import build as b
    b.build()


def _T(x):
    return torch.from_numpy(np.ascontiguousarray(x, np.float32)).to(DEV)


def _close(got, ref, name, rtol=1e-5, rows=None):
    got, ref = np.asarray(got), np.asarray(ref)
    if rows is not None:
        got, ref = got[rows], ref[rows]
    np.testing.assert_allclose(got, ref, rtol=rtol, atol=1e-6 * max(1.0, float(np.abs(ref).max())), err_msg=name)


def _last_sigma_agrees(sig_gpu, sig_ref):
    """Rays whose last-sample sigma is zero on both sides or positive on both."""
    return (np.asarray(sig_gpu)[:, -1] > 0) == (np.asarray(sig_ref)[:, -1] > 0)


def _render_inputs(n=1024):
    rng = np.random.default_rng(0)
    o = (rng.standard_normal((n, 3)) * 0.1).astype(np.float32)
    d = rng.standard_normal((n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    u_c = rng.random((n, 64), dtype=np.float32)
    u_f = rng.random((n, 128), dtype=np.float32)
    return o, d, u_c, u_f


def test_render_1024_rays_matches_oracle():
    """The 1024-ray render through the functional path (stratified z, PE + MLP,
    compositing, inverse-CDF fine z, fine pass) against the oracle's
    render_rays (SimpleNeRF17.py:159-328) on the same uniforms."""
    from simple_rf_gb300 import functional as F
    n = 1024
    o, d, u_c, u_f = _render_inputs(n)
    ospec = on.MlpSpec()
    pc, pf = on.xavier_params(ospec, 0), on.xavier_params(ospec, 1)
    spec = F.MlpSpec()
    vd = F.view_dirs(_T(d))
    got = {}
    with torch.no_grad():
        def run(p, z):
            s = z.shape[1]
            pts = (_T(o)[:, None, :] + _T(d)[:, None, :] * z[:, :, None]).reshape(-1, 3).contiguous()
            sigma, rgb = F.NerfMlpFunction.apply(spec, 0, pts, vd, s, None, *[_T(p[k]) for k in spec.param_names])
            out = F.composite(sigma.reshape(n, s), rgb.reshape(n, s, 3), z, _T(d))
            return out, sigma.reshape(n, s)
        zc = F.stratified_z(n, 64, 2.0, 6.0, _T(u_c), device=DEV)
        oc, sc = run(pc, zc)
        zf = F.fine_z(zc, oc['weights'], 128, _T(u_f))
        of, sf = run(pf, zf)
    for tag, out, sig, z in (('coarse', oc, sc, zc), ('fine', of, sf, zf)):
        for k in ('rgb', 'depth', 'weights', 'acc'):
            got[f'{k}_{tag}'] = out[k].cpu().numpy()
        got[f'sigma_{tag}'] = sig.cpu().numpy()
        got[f'z_{tag}'] = z.cpu().numpy()
    ref, _ = on.render_rays(pc, pf, ospec, ospec, o, d, 2.0, 6.0, 64, 128, u_c, u_f, z_fine=got['z_fine'],
                            pts_fp32=True)
    np.testing.assert_array_equal(got['z_coarse'], ref['z_vals_coarse'])
    # the oracle's own inverse-CDF depths: equal up to the conditioning of the
    # sampler (the kernel tests compare it in CDF space)
    zf_ref = on.fine_z(ref['z_vals_coarse'], ref['weights_coarse'], 128, u_f)
    frac = float(np.mean(np.abs(got['z_fine'] - zf_ref) <= 1e-5 * np.abs(zf_ref)))
    assert frac > 0.999, frac
    keep = _last_sigma_agrees(got['sigma_coarse'], ref['raw_sigma_coarse'][..., 0]) & \
        _last_sigma_agrees(got['sigma_fine'], ref['raw_sigma_fine'][..., 0])
    assert keep.mean() > 0.995, int((~keep).sum())
    for tag in ('coarse', 'fine'):
        for k in ('rgb', 'depth', 'weights', 'acc'):
            _close(got[f'{k}_{tag}'], ref[f'{k}_{tag}'], f'{k}_{tag}', rows=keep)
    print('1024-ray render: rays excluded for a last-sample sigma flip', int((~keep).sum()), 'of', n,
          '; fine depths equal to the oracle sampler', frac)


def test_drop_in_render_1024_rays_matches_oracle():
    """GbSimpleNeRF.forward in evaluation mode (linspace coarse depths,
    deterministic inverse CDF) on the same 1024 rays, ray generation patched to
    take the synthetic origins and directions as the reference harness does."""
    from simple_rf_gb300 import functional as F
    from simple_rf_gb300.nerf import GbSimpleNeRF
    mc = {'num_samples': 64, 'points_net_depth': 8, 'views_net_depth': 1, 'points_net_width': 256,
          'views_net_width': 128, 'points_positional_encoding_degree': 10, 'views_positional_encoding_degree': 4,
          'use_view_dirs': True, 'view_dependent_rgb': True, 'predict_visibility': False}
    configs = {'data_loader': {'ndc': False}, 'model': {
        'name': 'GbSimpleNeRF01', 'coarse_model': mc, 'fine_model': dict(mc, num_samples=128),
        'learn_camera_focal_length': False, 'learn_camera_rotation': False, 'learn_camera_translation': False,
        'chunk': 4096, 'lindisp': False, 'netchunk': 16384, 'perturb': False, 'raw_noise_std': 0.0,
        'white_bkgd': False}}
    model_configs = {'intrinsics': np.eye(3)[None], 'extrinsics': np.eye(4)[None], 'resolution': (32, 32),
                     'near': 2.0, 'far': 6.0, 'near_ndc': 0.0, 'far_ndc': 1.0}
    n = 1024
    o, d, _, _ = _render_inputs(n)
    model = GbSimpleNeRF(configs, model_configs).to(DEV).eval()
    spec = on.MlpSpec()
    pc, pf = on.xavier_params(spec, 0), on.xavier_params(spec, 1)
    with torch.no_grad():
        for mod, p in ((model.coarse_model, pc), (model.fine_model, pf)):
            for name, prm in mod.named_parameters():
                prm.copy_(torch.from_numpy(p[name]))
    model.generate_rays = lambda input_dict, mode: {'rays_o': _T(o), 'rays_d': _T(d), 'view_dirs': F.view_dirs(_T(d))}
    batch = {'pixel_id': torch.zeros(n, 3, dtype=torch.int32, device=DEV), 'num_frames': 1, 'common_data': {}}
    with torch.no_grad():
        ret = model(batch, retraw=True)
    got = {k: v.cpu().numpy() for k, v in ret.items() if isinstance(v, torch.Tensor)}
    ref, _ = on.render_rays(pc, pf, spec, spec, o, d, 2.0, 6.0, 64, 128, None, None, z_fine=got['z_vals_fine'],
                            pts_fp32=True)
    keep = _last_sigma_agrees(got['raw_sigma_coarse'][..., 0], ref['raw_sigma_coarse'][..., 0]) & \
        _last_sigma_agrees(got['raw_sigma_fine'][..., 0], ref['raw_sigma_fine'][..., 0])
    assert keep.mean() > 0.995, int((~keep).sum())
    _close(got['z_vals_coarse'], ref['z_vals_coarse'], 'z_vals_coarse', rtol=1e-6)
    for k in ('rgb_coarse', 'depth_coarse', 'weights_coarse', 'acc_coarse', 'rgb_fine', 'depth_fine',
              'weights_fine', 'acc_fine'):
        _close(got[k], ref[k], k, rows=keep)
    # the variance sums w (z - depth)^2 with (z - depth)^2 up to (far - near)^2 = 16, so
    # the weights' absolute floor of 1e-6 (last samples: delta = 1e10 |d|) becomes 1.6e-5
    for k in ('depth_var_coarse', 'depth_var_fine'):
        np.testing.assert_allclose(got[k][keep], ref[k][keep], rtol=1e-5, atol=1.6e-5, err_msg=k)


# ------------------------------------------------------ 4096-ray training step --

def _step(n_rays, precision='fp32', sigma_bias=None, seed=3):
    from simple_rf_gb300.train_step import NerfTrainStep, synthetic_batch
    step = NerfTrainStep(n_rays, 64, 128, precision=precision, device=DEV, seed=seed)
    if sigma_bias is not None:
        for net in step.nets.values():
            net.views[net.spec.param_names.index('pts_output_linear.bias')].fill_(sigma_bias)
    batch = synthetic_batch(n_rays, 64, 128, seed=seed + 1, device=DEV)
    step.set_batch(*batch)
    params = {tag: {k: v.double().cpu().numpy() for k, v in net.state_dict().items()} for tag, net in step.nets.items()}
    step.step()
    torch.cuda.synchronize()
    out = {k: v.detach().cpu().numpy() for k, v in step.outputs().items()}
    grads = {tag: {k: g.double().cpu().numpy() for k, g in zip(net.spec.param_names, net.gviews)}
             for tag, net in step.nets.items()}
    host = [x.cpu().numpy() for x in batch]
    return params, out, grads, host


def oracle_step_chunked(params, host, z_fine, dtype, chunk=256, grads=True):
    """The oracle's 4096-ray training step over ray chunks (rays are independent, so the
    outputs are those of one whole-batch call; the loss gradients come from the
    whole batch and the parameter gradients are summed over the chunks)."""
    o, d, t_rgb, t_depth, u_c, u_f = [np.asarray(x, dtype) for x in host]
    spec = on.MlpSpec()
    p = {tag: {k: v.astype(dtype) for k, v in params[tag].items()} for tag in params}
    n = o.shape[0]

    def fwd(sl):
        return on.render_rays(p['coarse'], p['fine'], spec, spec, o[sl], d[sl], 2.0, 6.0, 64, 128, u_c[sl], u_f[sl],
                              white_bkgd=True, z_fine=np.asarray(z_fine[sl], dtype), pts_fp32=True)
    parts = [fwd(slice(i, i + chunk))[0] for i in range(0, n, chunk)]
    ret = {k: np.concatenate([r[k] for r in parts], 0) for k in parts[0]}
    if not grads:
        return ret, None
    mask = np.zeros(n, dtype)
    mask[:n // 4] = 1
    _, g = on.train_loss(ret, t_rgb, t_depth, mask)
    total = None
    for i in range(0, n, chunk):
        sl = slice(i, i + chunk)
        _, caches = fwd(sl)
        gi = on.backward_render(p, {'coarse': spec, 'fine': spec}, caches, {k: v[sl] for k, v in g.items()},
                                sl.stop - sl.start)
        if total is None:
            total = {t: {k: v.astype(np.float64) for k, v in gt.items()} for t, gt in gi.items()}
        else:
            for t in gi:
                for k in gi[t]:
                    total[t][k] += gi[t][k]
        del caches
    return ret, total


def test_train_step_4096_rays_outputs_match_oracle():
    """The fused FP32 plain step at the benchmark's 4096 rays: coarse and fine
    rgb/depth/weights/acc against the float32 oracle (fine pass on the depths
    the GPU sampled), the Xavier-initialised nets as trained."""
    params, out, _, host = _step(4096)
    ref, _ = oracle_step_chunked(params, host, out['z_fine'], np.float32, chunk=512, grads=False)
    np.testing.assert_array_equal(out['z_coarse'], ref['z_vals_coarse'])
    keep = np.ones(4096, bool)
    for tag in ('coarse', 'fine'):
        keep &= _last_sigma_agrees(out[f'sigma_{tag}'].reshape(4096, -1), ref[f'raw_sigma_{tag}'][..., 0])
    assert keep.mean() > 0.995, int((~keep).sum())
    for tag in ('coarse', 'fine'):
        for k in ('rgb_map', 'depth', 'weights', 'acc'):
            key = {'rgb_map': 'rgb'}.get(k, k)
            _close(out[f'{k}_{tag}'], ref[f'{key}_{tag}'], f'{k}_{tag}', rows=keep)
    print('4096-ray step: rays excluded for a last-sample sigma flip', int((~keep).sum()), 'of 4096')


def test_train_step_4096_rays_gradients_match_fp64_oracle():
    """Parameter gradients of the 4096-ray FP32 plain step against the float64
    oracle, on a network whose sigma-head bias keeps every ray off the last-sample
    step (see test_gpu_train_step.py)."""
    from test_gpu_train_step import check_fp32_gradients
    params, out, grads, host = _step(4096, sigma_bias=0.5)
    _, g64 = oracle_step_chunked(params, host, out['z_fine'], np.float64)
    _, g32 = oracle_step_chunked(params, host, out['z_fine'], np.float32)
    check_fp32_gradients(grads, g32, g64)


# --------------------------------------------------------- TensoRF 300^3 --

def _oracle_params(tm):
    tp = {'bbox': tm.bounding_box.cpu().numpy().astype(np.float32)}
    for kind, plist in (('planes_density', tm.matrices_density), ('lines_density', tm.vectors_density),
                        ('planes_color', tm.matrices_color), ('lines_color', tm.vectors_color)):
        tp[kind] = [np.ascontiguousarray(p.detach()[0].cpu().numpy()) for p in plist]
    tp['basis_matrix_color.weight'] = tm.basis_matrix_color.weight.detach().cpu().numpy()
    for k, prm in tm.color_predictor.named_parameters():
        tp['color_predictor.' + k] = prm.detach().cpu().numpy()
    return tp


def _tensorf_run(n_rays, seed=21):
    from simple_rf_gb300 import functional as F
    from simple_rf_gb300.bench_tensorf import make_models, synthetic_rays
    tm = make_models(DEV, precision='fp32')[0]
    tm.eval()
    o, d, _, u = synthetic_rays(n_rays, seed, DEV)
    bbox, s, step = tm.host_geometry()
    assert (s, tuple(int(r) for r in tm.resolution)) == (1039, (300, 300, 300))
    z = F.aabb_z(o, d, s, bbox, 2.0, 6.0, step, u[:, 0].contiguous())
    vd = F.view_dirs(d)
    out = tm({'z_vals': z, 'rays_o': o, 'rays_d': d, 'view_dirs': vd}, retraw=True)
    return tm, (o, d, z), out


def _oracle_forward(tm, o, d, z):
    spec = ot.RendererSpec(features_dim=27, features_pe=2, views_pe=2, units=128)
    am = tm.alpha_mask
    return ot.tensorf_forward(_oracle_params(tm), spec, o, d, z, alpha_vol=am.volume().float().cpu().numpy(),
                              alpha_bbox=am.bounding_box.cpu().numpy().astype(np.float32), distance_scale=25.0,
                              weight_threshold=1e-4, white=True), spec


def _threshold_stable(w_gpu, w_ref, thr=1e-4):
    """Rays none of whose samples straddles the surface threshold between the two
    weight sets or lies within 1e-5 relative of it."""
    side = (w_gpu > thr) != (w_ref > thr)
    near = np.abs(w_ref - thr) <= 1e-5 * thr
    return ~(side | near).any(1)


def test_tensorf_300cubed_8192_rays_outputs_match_oracle():
    """The drop-in GbVmTensor at the benchmark's main model (300^3, R 16 / 48,
    27 features, 128 units, 128^3 alpha mask at 15%, white background, 1039
    samples per ray) on 8192 rays against the float32 oracle of
    LowRankTensor.forward (SimpleTensoRF09.py:701-761)."""
    tm, (o, d, z), out = _tensorf_run(8192)
    oh, dh, zh = (x.cpu().numpy() for x in (o, d, z))
    ref, _ = _oracle_forward(tm, oh, dh, zh)[0]
    got = {k: v.detach().cpu().numpy() for k, v in out.items()}
    keep = _threshold_stable(got['weights'], ref['weights'])
    n_surface = int((ref['weights'] > 1e-4).sum())
    assert n_surface > 100000, n_surface
    assert keep.mean() > 0.99, int((~keep).sum())
    for k in ('rgb', 'depth', 'acc', 'weights', 'depth_var', 'raw_sigma'):
        _close(got[k], ref[k], k, rows=keep)
    print('TensoRF 300^3: surface samples', n_surface, '; rays excluded at the surface threshold', int((~keep).sum()),
          'of 8192')


def test_tensorf_300cubed_gradients_match_oracle():
    """Gradients of every plane, line, basis and renderer parameter of the 300^3 TensoRF
    main model for a loss on 256 of the 8192 rays (the other rays carry zero
    cotangents, so the gradients are those of the 256 rays alone) against the
    float64 oracle's adjoint: per tensor within max(1e-4, 3 e32) relative L2, e32
    being the float32 oracle's own error on the same inputs.

    The 256 rays are the first ones with acc >= 0.05 (the depth of a nearly
    transparent ray is sum(w z) / (acc + 1e-6), whose gradient (z - depth) /
    (acc + 1e-6) amplifies rounding by up to 1e6, so such rays measure the
    conditioning of the reference formula rather than the kernels) that have no
    sample on the 1e-4 surface threshold between the GPU and the float64 oracle
    (a sample coloured on one side only adds a renderer term to one gradient),
    no density at their last sample (whose delta is 1e10 |d|) and no density
    feature within 1e-6 of the ReLU's kink."""
    tm, (o, d, z), out = _tensorf_run(8192, seed=22)
    n_sub = 256
    spec = ot.RendererSpec(features_dim=27, features_pe=2, views_pe=2, units=128)
    am = tm.alpha_mask
    tp32 = _oracle_params(tm)

    def oracle(rows, dt):
        cast = {k: ([a.astype(dt) for a in v] if isinstance(v, list) else v.astype(dt)) for k, v in tp32.items()}
        oh, dh, zh = (x[rows].cpu().numpy().astype(dt) for x in (o, d, z))
        return ot.tensorf_forward(cast, spec, oh, dh, zh, alpha_vol=am.volume().float().cpu().numpy().astype(dt),
                                  alpha_bbox=am.bounding_box.cpu().numpy().astype(dt), distance_scale=25.0,
                                  weight_threshold=1e-4, white=True), cast

    # candidate rays: opaque enough, and no sample on the surface threshold between
    # this float32 evaluation and the float64 one
    acc = out['acc'].detach().cpu().numpy()
    cand = np.nonzero(acc >= 0.05)[0][:2 * n_sub]
    (ref_c, _), _ = oracle(cand, np.float64)
    stable = _threshold_stable(out['weights'][cand].detach().cpu().numpy(), ref_c['weights'])
    # and no density at the last sample: its delta is 1e10 |d| (SimpleTensoRF09.py:787-791),
    # so a positive last sigma that sits within rounding of 0 (a density feature summed
    # to ~0 from terms of ~1e-3) has a gradient of ~1e13 that the two evaluations of
    # that feature decide, not the kernels
    last = out['raw_sigma'][cand, -1, 0].detach().cpu().numpy()
    stable &= (last == 0) & (ref_c['raw_sigma'][:, -1, 0] == 0)
    # and no valid sample whose density feature lies within rounding of the ReLU's
    # kink (a sum of 48 products of ~1e-2 that cancels to below 1e-6): the two
    # evaluations may put it on different sides, adding its term to one gradient only
    (_, cache_c), _ = oracle(cand, np.float64)
    s_per_ray = z.shape[1]
    kink_rays = np.unique(cache_c['vflat'][np.abs(cache_c['sig_feat']) < 1e-6] // s_per_ray)
    stable[kink_rays] = False
    rows = cand[stable][:n_sub]
    assert rows.size == n_sub and stable.mean() > 0.9, (rows.size, stable.mean())
    rng = np.random.default_rng(5)
    cot = {k: np.zeros(tuple(out[k].shape), np.float32) for k in ('rgb', 'depth', 'acc')}
    for k in cot:
        cot[k][rows] = rng.standard_normal(cot[k][rows].shape).astype(np.float32)
    loss = sum((out[k] * _T(cot[k])).sum() for k in cot)
    loss.backward()
    grads = {}
    for dt in (np.float64, np.float32):
        (ref, cache), cast = oracle(rows, dt)
        grads[dt] = ot.tensorf_backward(cast, spec, cache, {k: v[rows].astype(dt) for k, v in cot.items()})
    pairs = []
    for kind, plist in (('planes_density', tm.matrices_density), ('lines_density', tm.vectors_density),
                        ('planes_color', tm.matrices_color), ('lines_color', tm.vectors_color)):
        for i in range(3):
            pairs.append((f'{kind}.{i}', plist[i].grad[0]))
    pairs.append(('basis_matrix_color.weight', tm.basis_matrix_color.weight.grad))
    for k, prm in tm.color_predictor.named_parameters():
        pairs.append(('color_predictor.' + k, prm.grad))
    worst = 0.0
    for name, grad in pairs:
        g64 = grads[np.float64][name].astype(np.float64)
        nrm = max(np.linalg.norm(g64), 1e-30)
        rel = np.linalg.norm(grad.detach().double().cpu().numpy() - g64) / nrm
        e32 = np.linalg.norm(grads[np.float32][name].astype(np.float64) - g64) / nrm
        bar = max(1e-4, 3 * e32)
        worst = max(worst, rel / bar)
        assert rel < bar, (name, rel, e32)
    print('TensoRF 300^3: worst per-tensor gradient error / bar', worst)


def _pair_oracle_forward(params, host, z_fine, dtype, chunk=512):
    """The oracle's forward of the NDC main + augmented pair (NDC, main coarse + fine, the
    augmented coarse net on the same coarse samples) over ray chunks."""
    o, d, _, _, u_c, u_f = [np.asarray(x, dtype) for x in host]
    spec = on.MlpSpec()
    aspec = on.MlpSpec(points_pe_degree=4, use_view_dirs=False, view_dependent_rgb=False)
    p = {tag: {k: v.astype(dtype) for k, v in params[tag].items()} for tag in params}
    aug = 'views_augmentation'
    parts = []
    for i in range(0, o.shape[0], chunk):
        sl = slice(i, min(i + chunk, o.shape[0]))
        focal = np.full(sl.stop - sl.start, 400.0, dtype)
        ret, _ = on.render_rays(p['coarse'], p['fine'], spec, spec, o[sl], d[sl], 0.0, 1.0, 64, 128, u_c[sl], u_f[sl],
                                ndc=dict(h=378, w=504, fx=focal, fy=focal, near=1.0),
                                aug=[(aug, {'coarse': p[f'{aug}_coarse']}, aspec)],
                                z_fine=np.asarray(z_fine[sl], dtype), pts_fp32=True)
        parts.append(ret)
    n0 = min(chunk, o.shape[0])
    keys = [k for k, v in parts[0].items() if isinstance(v, np.ndarray) and v.ndim >= 1 and v.shape[0] == n0]
    return {k: np.concatenate([r[k] for r in parts], 0) for k in keys}


@pytest.mark.parametrize('precision', ['fp32', 'fp16'])
def test_ndc_pair_step_4096_rays_matches_oracle(precision):
    """The NDC pair step (main coarse + fine + augmented coarse, 4096
    rays) against the oracle: FP32 plain rgb / weights / acc within 1e-5 of the
    float32 oracle (acc with one ulp(1) per sample), the NDC depth within 1e-5 of
    the float64 reduction of the GPU's own weights; the FP16 step's
    rgb within 2e-3 max-abs of the float64 oracle.  NDC rays end at z = 1 (no
    1e10 last delta), so no ray is excluded."""
    from simple_rf_gb300.train_step import make_step
    aug = 'views_augmentation'
    step, batch_fn = make_step('nerf_pair', 4096, precision, DEV, seed=5)
    batch = batch_fn(6, DEV)
    step.set_batch(*batch)
    params = {tag: {k: v.double().cpu().numpy() for k, v in net.state_dict().items()} for tag, net in step.nets.items()}
    step.step()
    torch.cuda.synchronize()
    out = {k: v.detach().cpu().numpy() for k, v in step.outputs().items()}
    host = [x.cpu().numpy() for x in batch]
    dtype = np.float32 if precision == 'fp32' else np.float64
    ref = _pair_oracle_forward(params, host, out['z_fine'], dtype)

    def key(k, tag):
        k = {'rgb_map': 'rgb'}.get(k, k)
        return f'{aug}_{k}_coarse' if tag.startswith(aug) else f'{k}_{tag}'

    worst = {}
    for tag in ('coarse', 'fine', f'{aug}_coarse'):
        if precision == 'fp32':
            for k in ('rgb_map', 'weights', 'acc'):
                r = ref[key(k, tag)]
                atol = out[f'weights_{tag}'].shape[1] * 2.0 ** -23 if k == 'acc' else \
                    1e-6 * max(1.0, float(np.abs(r).max()))
                np.testing.assert_allclose(out[f'{k}_{tag}'], r, rtol=1e-5, atol=atol, err_msg=f'{k}_{tag}')
            # depth_ndc = sum w z / (acc + 1e-6) divides by acc, whose absolute rounding
            # (one ulp(1) per sample) is large relative to a small acc: the weights are
            # compared above, the depth as the float64 reduction of the GPU's weights
            w = out[f'weights_{tag}'].astype(np.float64)
            zr = np.sum(w * out[f'z_{tag}'].astype(np.float64), -1) / (np.sum(w, -1) + 1e-6)
            np.testing.assert_allclose(out[f'depth_ndc_{tag}'], zr, rtol=1e-5, atol=1e-6, err_msg=f'depth_ndc_{tag}')
        else:
            worst[tag] = float(np.abs(out[f'rgb_map_{tag}'] - ref[key('rgb_map', tag)]).max())
            assert worst[tag] < 2e-3, (tag, worst[tag])
    if worst:
        print('fp16 pair step, 4096 rays: rgb max-abs vs float64', worst)


def test_full_view_render_504x378_matches_oracle():
    """One full view of the image render (504 x 378 = 190,512 NDC rays, focal 400) through the
    FP32 plain pair renderer in chunks of 65,536 (the last chunk partial): rays at
    the start, across the first chunk boundary and in the partial last chunk
    against the float32 oracle (rgb and acc of the three nets within 1e-5
    relative plus one ulp(1) per sample absolute; the fine pass on the depths the
    GPU sampled)."""
    from simple_rf_gb300.render import NerfPairRenderer, pixel_rays, synthetic_views
    aug = 'views_augmentation'
    pid, intr, ext = synthetic_views(1, 378, 504, focal=400.0, seed=9, device=DEV)
    o, d = pixel_rays(pid, intr, ext)
    n = o.shape[0]
    r = NerfPairRenderer(65536, 'fp32', DEV, seed=4, graph=False)
    out = r.render(o, d, keep=('rgb', 'acc', 'z'))
    torch.cuda.synchronize()
    assert n == 190512 and out['coarse']['rgb'].shape[0] == n
    sel = np.concatenate([np.arange(0, 256), np.arange(65536 - 256, 65536 + 256), np.arange(n - 512, n)])
    params = {tag: {k: v.cpu().numpy() for k, v in net.state_dict().items()} for tag, net in r.nets.items()}
    spec = on.MlpSpec()
    aspec = on.MlpSpec(points_pe_degree=4, use_view_dirs=False, view_dependent_rgb=False)
    focal = np.full(sel.size, 400.0, np.float32)
    ret, _ = on.render_rays(params['coarse'], params['fine'], spec, spec, o.cpu().numpy()[sel], d.cpu().numpy()[sel],
                            0.0, 1.0, 64, 128, ndc=dict(h=378, w=504, fx=focal, fy=focal, near=1.0),
                            aug=[(aug, {'coarse': params[f'{aug}_coarse']}, aspec)],
                            z_fine=out['fine']['z'].cpu().numpy()[sel])
    for tag, pre in (('coarse', ''), ('fine', ''), (f'{aug}_coarse', f'{aug}_')):
        lvl = 'fine' if tag == 'fine' else 'coarse'
        n_s = out[tag]['z'].shape[1]
        for k in ('rgb', 'acc'):
            # rgb = sum w c and acc = sum w: each weight carries an absolute rounding of
            # up to ulp(1) = 2^-23 (1 - alpha, the transmittance products), colours <= 1
            np.testing.assert_allclose(out[tag][k].cpu().numpy()[sel], ret[f'{pre}{k}_{lvl}'], rtol=1e-5,
                                       atol=n_s * 2.0 ** -23, err_msg=f'{k}_{tag}')
