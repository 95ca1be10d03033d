"""The drop-in TensoRF VM model (CUDA path) against the reference's own outputs and
autograd gradients (golden fixture produced by tests/golden/make_golden.py from
SimpleTensoRF09.LowRankTensor.forward), and against the numpy oracle.

Tolerances: outputs 1e-5 relative (absolute floor 1e-6 of the value range);
parameter gradients 1e-4 relative L2.  A sample whose weight lies within float32
rounding of the 1e-4 surface threshold (SimpleTensoRF09.py:726) may be coloured
by one implementation and not the other: rays holding such a sample are left out
of the output comparison and counted (at most 1% of the rays), and when any ray
was left out the gradient bar becomes 1e-3 (the flipped sample's colour term is
in one gradient only).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = 'cuda'


def _tcfg():
    return {'decomposition_type': 'VectorMatrix', 'num_samples_max': 1e6, 'num_components_density': [4, 3, 2],
            'num_components_color': [6, 5, 4], 'bounding_box': [[-1.5] * 3, [1.5] * 3],
            'num_voxels_initial': 20 * 22 * 24, 'num_voxels_final': 20 * 22 * 24, 'tensor_upsampling_iters': [],
            'num_voxels_per_sample': 0.5, 'alpha_mask_update_iters': [], 'alpha_mask_threshold': 1e-4,
            'ray_marching_weight_threshold': 1e-4, 'use_view_dirs': True, 'view_dependent_color': True,
            'views_positional_encoding_degree': 2, 'features_positional_encoding_degree': 2,
            'features_dimension_color': 7, 'density_offset': -10, 'distance_scale': 25, 'density_predictor': 'ReLU',
            'color_predictor': 'MLP_Features', 'num_units_color_predictor': 16, 'predict_visibility': False}


def _model(g, ndc=False):
    from simple_rf_gb300 import build as b
    b.build()
    from simple_rf_gb300 import tensorf as T
    from simple_rf_gb300.tensorf_model import AlphaGridMask, GbVmTensor
    configs = {'data_loader': {'ndc': ndc}, 'model': {'white_bkgd': not ndc}}
    tcfg = dict(_tcfg(), bounding_box=g['bbox'].tolist())
    tm = GbVmTensor('coarse_model', configs, tcfg, {'bounding_box': tcfg['bounding_box']})
    tm.update_tensor_params(torch.tensor(g['res']), torch.tensor(g['bbox']))
    with torch.no_grad():
        for kind, plist in (('planes_density', tm.matrices_density), ('lines_density', tm.vectors_density),
                            ('planes_color', tm.matrices_color), ('lines_color', tm.vectors_color)):
            for i in range(3):
                plist[i] = torch.nn.Parameter(T.to_channels_last(torch.from_numpy(g[f'{kind}.{i}'])[None]))
        tm.basis_matrix_color.weight.copy_(torch.from_numpy(g['basis_matrix_color.weight']))
        for k, prm in tm.color_predictor.named_parameters():
            prm.copy_(torch.from_numpy(g['color_predictor.' + k]))
    tm = tm.to(DEV)
    tm.alpha_mask = AlphaGridMask(torch.from_numpy(g['alpha_vol']).to(DEV), torch.tensor(g['bbox']).to(DEV))
    tm.eval()
    return tm


def threshold_stable(w_gpu, w_ref, thr=1e-4):
    """Rays none of whose samples has weights on both sides of the surface
    threshold between the two implementations, or within 1e-5 relative of it."""
    side = (w_gpu > thr) != (w_ref > thr)
    near = np.abs(w_ref - thr) <= 1e-5 * thr
    return ~(side | near).any(-1)


def compare_outputs(out, g, keys):
    """Outputs against the golden on the threshold-stable rays; returns the
    gradient bar (1e-4, or 1e-3 when a ray was left out)."""
    keep = threshold_stable(out['weights'].detach().cpu().numpy(), g['out_weights'])
    assert keep.mean() >= 0.99 or keep.sum() >= keep.size - 1, int((~keep).sum())
    for k in keys:
        ref = g['out_' + k][keep]
        got = out[k].detach().cpu().numpy()[keep]
        np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6 * max(1.0, float(np.abs(ref).max())), err_msg=k)
    return 1e-4 if keep.all() else 1e-3


def compare_gradients(tm, g, bar):
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
        ref = g['grad_' + name]
        got = grad.detach().double().cpu().numpy()
        rel = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
        worst = max(worst, rel)
        assert rel < bar, (name, rel)
    return worst


def test_tensorf_forward_backward_matches_reference_golden(golden):
    g = golden('tensorf')
    tm = _model(g)
    o = torch.from_numpy(g['rays_o']).to(DEV)
    d = torch.from_numpy(g['rays_d']).to(DEV)
    z = torch.from_numpy(g['z']).to(DEV)
    vd = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    out = tm({'z_vals': z, 'rays_o': o, 'rays_d': d, 'view_dirs': vd}, retraw=True)
    bar = compare_outputs(out, g, ('rgb', 'depth', 'acc', 'weights', 'raw_sigma', 'depth_var'))
    loss = sum((out[k] * torch.from_numpy(g[f'cot_{k}']).to(DEV)).sum() for k in ('rgb', 'depth', 'acc'))
    loss.backward()
    compare_gradients(tm, g, bar)


def test_tensorf_ndc_forward_backward_matches_reference_golden(golden):
    """NDC mode (the forward-facing TensoRF configuration): samples march along
    the NDC rays, compositing takes NDC deltas and converts depths with the world
    rays; outputs and gradients against the reference's LowRankTensor.forward
    (golden tensorf_ndc, no white background: the coin came up >= 0.5)."""
    g = golden('tensorf_ndc')
    tm = _model(g, ndc=True)
    tm.eval()
    t = {k: torch.from_numpy(g[k]).to(DEV) for k in ('rays_o', 'rays_d', 'rays_o_ndc', 'rays_d_ndc', 'view_dirs', 'z')}
    out = tm({'z_vals_ndc': t['z'], 'rays_o_ndc': t['rays_o_ndc'], 'rays_d_ndc': t['rays_d_ndc'],
              'rays_o': t['rays_o'], 'rays_d': t['rays_d'], 'view_dirs': t['view_dirs']}, retraw=True)
    bar = compare_outputs(out, g, ('rgb', 'depth', 'depth_ndc', 'acc', 'weights', 'raw_sigma', 'depth_var',
                                   'depth_var_ndc'))
    loss = sum((out[k] * torch.from_numpy(g[f'cot_{k}']).to(DEV)).sum() for k in ('rgb', 'depth', 'depth_ndc', 'acc'))
    loss.backward()
    compare_gradients(tm, g, bar)


def test_tensorf_realistic_model_matches_reference_golden(golden):
    """The drop-in GbVmTensor at the benchmark's model shape on a 48^3 grid (16 / 48
    components, 27 features, 128 renderer units, PE L=2, a 32^3 alpha mask at 15%,
    white background, 256 rays) against LowRankTensor.forward's outputs and
    autograd gradients (golden tensorf_realistic)."""
    from oracle import tensorf as ot
    from simple_rf_gb300 import tensorf as T
    from simple_rf_gb300.tensorf_model import AlphaGridMask, GbVmTensor
    g = golden('tensorf_realistic')
    c = {k[4:]: g[k] for k in g if k.startswith('cfg_')}
    tp, _ = ot.seeded_vm_model(int(c['seed']), [int(c['res'])] * 3, list(c['density']), list(c['color']),
                               int(c['features']), int(c['units']))
    tcfg = dict(_tcfg(), num_components_density=[int(x) for x in c['density']],
                num_components_color=[int(x) for x in c['color']], num_voxels_initial=int(c['res']) ** 3,
                num_voxels_final=int(c['res']) ** 3, features_dimension_color=int(c['features']),
                num_units_color_predictor=int(c['units']))
    tm = GbVmTensor('coarse_model', {'data_loader': {'ndc': False}, 'model': {'white_bkgd': True}}, tcfg,
                    {'bounding_box': tcfg['bounding_box']})
    assert [int(r) for r in tm.resolution] == [int(c['res'])] * 3
    with torch.no_grad():
        for kind, mats, vecs in (('density', tm.matrices_density, tm.vectors_density),
                                 ('color', tm.matrices_color, tm.vectors_color)):
            for i in range(3):
                mats[i] = torch.nn.Parameter(T.to_channels_last(torch.from_numpy(tp[f'planes_{kind}'][i])[None]))
                vecs[i] = torch.nn.Parameter(T.to_channels_last(torch.from_numpy(tp[f'lines_{kind}'][i])[None]))
        tm.basis_matrix_color.weight.copy_(torch.from_numpy(tp['basis_matrix_color.weight']))
        for k, prm in tm.color_predictor.named_parameters():
            prm.copy_(torch.from_numpy(tp['color_predictor.' + k]))
    tm = tm.to(DEV)
    tm.alpha_mask = AlphaGridMask(torch.from_numpy(g['alpha_vol'].astype(np.float32)).to(DEV),
                                  torch.tensor(g['bbox']).to(DEV))
    tm.eval()
    o, d, z = (torch.from_numpy(g[k]).to(DEV) for k in ('rays_o', 'rays_d', 'z'))
    vd = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    out = tm({'z_vals': z, 'rays_o': o, 'rays_d': d, 'view_dirs': vd}, retraw=True)
    assert tm.last_sample_counts['surface'] > 5000
    bar = compare_outputs(out, g, ('rgb', 'depth', 'acc', 'weights', 'raw_sigma', 'depth_var'))
    loss = sum((out[k] * torch.from_numpy(g[f'cot_{k}']).to(DEV)).sum() for k in ('rgb', 'depth', 'acc'))
    loss.backward()
    print('realistic golden: worst gradient rel-L2', compare_gradients(tm, g, bar))


def test_tensorf_aabb_marching_matches_reference(golden):
    from simple_rf_gb300 import functional as F
    g = golden('tensorf')
    z = F.aabb_z(torch.from_numpy(g['rays_o']).to(DEV), torch.from_numpy(g['rays_d']).to(DEV),
                 int(g['num_samples']), g['bbox'], 0.5, 6.0, float(g['step_size']),
                 torch.from_numpy(g['u']).to(DEV))
    np.testing.assert_allclose(z.cpu().numpy(), g['z'], rtol=1e-6, atol=1e-6)


def test_tensorf_full_size_grid_gather_roundtrip():
    """300^3-class grid with R = 16/48 components (the benchmark shape): the VM
    density gather is linear in the planes, so scaling every plane by 2 doubles
    the features exactly (size-independent property at full size)."""
    from simple_rf_gb300 import tensorf as T
    torch.manual_seed(0)
    res = [300, 300, 300]
    planes = [T.to_channels_last(torch.randn(1, 16, 300, 300, device=DEV) * 0.1) for _ in range(3)]
    lines = [T.to_channels_last(torch.randn(1, 16, 300, 1, device=DEV) * 0.1) for _ in range(3)]
    pts = torch.rand(1 << 20, 3, device=DEV) * 2 - 1
    f1 = T.vm_density(T.VmGridTensors(planes, lines, res), pts)
    f2 = T.vm_density(T.VmGridTensors([p * 2 for p in planes], lines, res), pts)
    assert torch.equal(f2, 2 * f1)
    cp = [T.to_channels_last(torch.randn(1, 48, 300, 300, device=DEV) * 0.1) for _ in range(3)]
    cl = [T.to_channels_last(torch.randn(1, 48, 300, 1, device=DEV) * 0.1) for _ in range(3)]
    c1 = T.vm_color(T.VmGridTensors(cp, cl, res), pts[:4096])
    assert c1.shape == (4096, 144) and torch.isfinite(c1).all()


@pytest.mark.parametrize('precision,bar,basis', [('fp16', 3e-2, None), ('bf16', 8e-2, None), ('fp16', 3e-2, 0),
                                                  ('fp16', 3e-2, 5)])
def test_tensorf_tensor_core_renderer_against_fp32(precision, bar, basis):
    """The 16-bit tensor-core renderer (basis + MlpFeaturesColorPredictor) against
    the FP32 path on the same model and rays (64^3 grid, R = 16/48, 128 units):
    rgb within 2e-3 max-abs; whole gradient of the renderer and the colour grid
    within `bar` relative L2.  `basis` pins the basis pass's tuned choice (0: the
    SIMT tile 2 x 128, 5: the TF32 tensor-core GEMM; None: what the tuner picks)."""
    from simple_rf_gb300 import _lib, autotune, build as b
    b.build()
    from simple_rf_gb300.bench_tensorf import make_models, synthetic_rays
    from simple_rf_gb300 import functional as F
    res = {}
    for prec in ('fp32', precision):
        tm = make_models(DEV, seed=3, precision=prec, grids=(64, 32))[0]
        o, d, t_rgb, u = synthetic_rays(256, 5, DEV)
        s = int(tm.num_samples.item())
        z = F.aabb_z(o, d, s, tm.bounding_box.detach().cpu(), 2.0, 6.0, float(tm.step_size), u[:, 0].contiguous())
        inp = {'z_vals': z, 'rays_o': o, 'rays_d': d, 'view_dirs': F.view_dirs(d)}
        if prec != 'fp32' and basis is not None:
            with torch.no_grad():
                tm(inp, retraw=False)      # the tuner records the basis site's key
            keys = [e['key'] for e in autotune.table() if e['site'] == 2]
            assert keys
            for k in keys:
                _lib.check(_lib.load().srf_autotune_set(2, *k, basis), 'srf_autotune_set')
        out = tm(inp, retraw=False)
        loss = ((out['rgb'] - t_rgb) ** 2).mean()
        loss.backward()
        params = [tm.basis_matrix_color.weight] + list(tm.color_predictor.parameters()) + list(tm.matrices_color) + \
            list(tm.vectors_color)
        groups = {'basis': [tm.basis_matrix_color.weight], 'mlp': list(tm.color_predictor.parameters()),
                  'colour_grid': list(tm.matrices_color) + list(tm.vectors_color)}
        res[prec] = (out['rgb'].detach(), torch.cat([p.grad.reshape(-1) for p in params]), tm.last_sample_counts,
                     {k: torch.cat([p.grad.reshape(-1) for p in v]) for k, v in groups.items()})
    (r32, g32, c32, p32), (r16, g16, c16, p16) = res['fp32'], res[precision]
    assert c32['surface'] > 1000 and c32 == c16, (c32, c16)
    err = (r16 - r32).abs().max().item()
    rel = ((g16 - g32).norm() / g32.norm()).item()
    # each group on its own: the basis weights (dB^T feats) and the colour grid
    # (through d_feats = dB . Wb) separate the two products of the basis adjoint
    per = {k: ((p16[k] - p32[k]).norm() / p32[k].norm()).item() for k in p32}
    print(precision, 'basis choice', basis, 'rgb max-abs', err, 'renderer+colour-grid gradient rel-L2', rel,
          'per group', per)
    if basis is not None:
        autotune.clear()
    assert err < 2e-3, err
    assert rel < bar, rel
    for k, v in per.items():
        assert v < bar, (k, v)


def test_tensorf_cp_matches_reference_golden(golden):
    """The CP decomposition (GbCpTensor on the CP lookup kernels) against
    CpDecomposedTensor's own outputs and autograd gradients (golden tensorf_cp)."""
    g = golden('tensorf_cp')
    from simple_rf_gb300 import build as b
    b.build()
    from simple_rf_gb300 import tensorf as T
    from simple_rf_gb300.tensorf_model import GbCpTensor, make_tensor_model
    tc = dict(_tcfg())
    tc.update(decomposition_type='CandecompParafac', num_components_density=[5], num_components_color=[6])
    configs = {'data_loader': {'ndc': False}, 'model': {'white_bkgd': True}}
    tm = make_tensor_model('coarse_model', configs, tc, {'bounding_box': tc['bounding_box']})
    assert isinstance(tm, GbCpTensor)
    tm.update_tensor_params(torch.tensor(g['res']), torch.tensor(g['bbox']))
    with torch.no_grad():
        for kind, plist in (('lines_density', tm.vectors_density), ('lines_color', tm.vectors_color)):
            for i in range(3):
                plist[i] = torch.nn.Parameter(T.to_channels_last(torch.from_numpy(g[f'{kind}.{i}'])[None]))
        tm.basis_matrix_color.weight.copy_(torch.from_numpy(g['basis_matrix_color.weight']))
        for k, prm in tm.color_predictor.named_parameters():
            prm.copy_(torch.from_numpy(g['color_predictor.' + k]))
    tm = tm.to(DEV)
    tm.eval()
    o = torch.from_numpy(g['rays_o']).to(DEV)
    d = torch.from_numpy(g['rays_d']).to(DEV)
    z = torch.from_numpy(g['z']).to(DEV)
    vd = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    out = tm({'z_vals': z, 'rays_o': o, 'rays_d': d, 'view_dirs': vd}, retraw=True)
    for k in ('rgb', 'depth', 'acc', 'weights', 'raw_sigma', 'depth_var'):
        ref = g['out_' + k]
        got = out[k].detach().cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=1e-4, atol=2e-4 * max(1.0, float(np.abs(ref).max())), err_msg=k)
    loss = sum((out[k] * torch.from_numpy(g[f'cot_{k}']).to(DEV)).sum() for k in ('rgb', 'depth', 'acc'))
    loss.backward()
    pairs = [(f'lines_density.{i}', tm.vectors_density[i].grad[0]) for i in range(3)]
    pairs += [(f'lines_color.{i}', tm.vectors_color[i].grad[0]) for i in range(3)]
    pairs.append(('basis_matrix_color.weight', tm.basis_matrix_color.weight.grad))
    for k, prm in tm.color_predictor.named_parameters():
        pairs.append(('color_predictor.' + k, prm.grad))
    for name, grad in pairs:
        ref = g['grad_' + name]
        rel = np.linalg.norm(grad.detach().cpu().numpy() - ref) / max(np.linalg.norm(ref), 1e-30)
        assert rel < 1e-3, (name, rel)


def _grads(step):
    return [p.grad.detach().double().clone() for p, _ in step.params]


def _rel(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b).clamp_min(1e-30))


@pytest.mark.parametrize('precision', ['fp32', 'fp16'])
def test_graph_step_matches_eager_step(precision):
    """The TensoRF training step captured as a CUDA graph (capacity-sized
    compacted launches) against the uncaptured step, from the same models on
    three batches: losses within 1e-5 relative, parameter gradients within 1e-4
    relative L2 per tensor (only the grouping of sums over samples differs).
    Learning rates are 0, so both steps see the same parameters at every call:
    with updates, Adam turns last-bit gradient differences of near-zero entries
    into +-lr steps and the runs drift apart (the update itself is covered by the
    overflow / re-capture tests below)."""
    from simple_rf_gb300 import build as b
    b.build()
    from simple_rf_gb300.bench_tensorf import TensorfGraphStep, TensorfTrainStep, make_models, synthetic_rays
    ea = TensorfTrainStep(make_models(DEV, seed=3, precision=precision, grids=(64, 32)), lr_tensor=0.0,
                          lr_network=0.0)
    gb = TensorfGraphStep(make_models(DEV, seed=3, precision=precision, grids=(64, 32)), 2048, lr_tensor=0.0,
                          lr_network=0.0)
    for i in range(3):
        batch = synthetic_rays(2048, 40 + i, DEV)
        la = float(ea.step(*batch).item())
        lb = float(gb.step(*batch).item())
        assert abs(la - lb) <= 1e-5 * abs(la), (i, la, lb)
        ga, gg = _grads(ea), _grads(gb)
        for (p, _), x, y in zip(ea.params, ga, gg):
            assert _rel(y, x) < 1e-4, (i, tuple(p.shape), _rel(y, x))
    counts = gb.sample_counts()
    assert [c['surface'] for c in counts] == [c['surface'] for c in ea.last['samples']]
    assert int(gb.step_dev.item()) == 3


def test_graph_step_redoes_a_step_that_overflowed():
    """Capacities below the sample counts: the replay raises the overflow flag
    and skips its update; the call re-captures with larger capacities and redoes
    the batch, so it returns what the uncaptured step computes: the first call's
    loss within 1e-5 and gradients within 1e-4 per tensor; the second call starts
    from parameters that Adam moved, where last-bit gradient differences of
    near-zero entries become +-lr steps, so its loss is held to 1e-4 and its
    gradients to 1e-2 relative L2 over all tensors."""
    from simple_rf_gb300 import build as b
    b.build()
    from simple_rf_gb300.bench_tensorf import TensorfGraphStep, TensorfTrainStep, make_models, synthetic_rays
    ea = TensorfTrainStep(make_models(DEV, seed=4, precision='fp32', grids=(64, 32)))
    gb = TensorfGraphStep(make_models(DEV, seed=4, precision='fp32', grids=(64, 32)), 2048)
    gb.MARGIN = 0.5   # the first capture is sized at half the counts
    for i in range(2):
        batch = synthetic_rays(2048, 50 + i, DEV)
        la = float(ea.step(*batch).item())
        lb = float(gb.step(*batch).item())
        assert abs(la - lb) <= (1e-5 if i == 0 else 1e-4) * abs(la), (i, la, lb)
        ga, gg = _grads(ea), _grads(gb)
        if i == 0:
            for (p, _), x, y in zip(ea.params, ga, gg):
                assert _rel(y, x) < 1e-4, (i, tuple(p.shape), _rel(y, x))
        else:
            whole = _rel(torch.cat([y.ravel() for y in gg]), torch.cat([x.ravel() for x in ga]))
            assert whole < 1e-2, (i, whole)
    assert gb.recaptures >= 1 and int(gb.flags_host[0]) == 0 and int(gb.step_dev.item()) == 2


def test_graph_step_shrinks_oversized_capacities():
    """Capacities three times the counts (the window of recent replays set to 2):
    after two calls the third re-captures at 15% above the largest recent counts;
    every call returns what the uncaptured step computes.  Learning rates are 0,
    so both steps see the same parameters at every call (with updates, Adam turns
    last-bit gradient differences into +-lr steps and the runs drift apart)."""
    from simple_rf_gb300 import build as b
    b.build()
    from simple_rf_gb300.bench_tensorf import TensorfGraphStep, TensorfTrainStep, make_models, synthetic_rays
    ea = TensorfTrainStep(make_models(DEV, seed=4, precision='fp32', grids=(64, 32)), lr_tensor=0.0, lr_network=0.0)
    gb = TensorfGraphStep(make_models(DEV, seed=4, precision='fp32', grids=(64, 32)), 2048, lr_tensor=0.0,
                          lr_network=0.0)
    gb.MARGIN = 3.0
    gb._recent = __import__('collections').deque(maxlen=2)
    for i in range(3):
        batch = synthetic_rays(2048, 60 + i, DEV)
        la = float(ea.step(*batch).item())
        lb = float(gb.step(*batch).item())
        assert gb.shrinks == (1 if i == 2 else 0), (i, gb.shrinks)
        assert abs(la - lb) <= 1e-5 * abs(la), (i, la, lb)
        for (p, _), x, y in zip(ea.params, _grads(ea), _grads(gb)):
            assert _rel(y, x) < 1e-4, (i, tuple(p.shape), _rel(y, x))
    counts = gb._host_counts()
    assert gb.shrinks == 1 and gb.recaptures == 0, (gb.shrinks, gb.recaptures)
    # re-captured from the recent maxima: at least the last counts, far below the initial 3x
    for (cv, cs), (nv, ns) in zip(gb.caps, counts):
        assert nv <= cv <= 2.0 * max(nv, gb.ROUND) and ns <= cs <= 2.0 * max(ns, gb.ROUND), (gb.caps, counts)


def test_alpha_mask_rebuild_matches_reference(golden):
    """LowRankTensor.update_alpha_mask (SimpleTensoRF09.py:849-876) on the drop-in:
    dense alpha of the density over the grid (the VM density kernel), 3^3 max-pool,
    threshold, and the occupied box, against the reference's (golden
    tensorf_maintenance: a density confined to a window of a 20 x 22 x 24 grid).
    A voxel whose pooled alpha sits on the 1e-4 threshold may switch sides between
    float32 evaluations: at most 0.1% of the volume may differ, and the box by at
    most one voxel."""
    from simple_rf_gb300 import build as b
    b.build()
    from simple_rf_gb300 import tensorf as T
    from simple_rf_gb300.tensorf_model import GbVmTensor
    g = golden('tensorf_maintenance')
    bbox = g['bbox'].tolist()
    tcfg = dict(_tcfg(), bounding_box=bbox, num_voxels_initial=int(np.prod(g['res'])),
                num_voxels_final=int(np.prod(g['res'])), num_components_density=[4, 3, 2],
                num_components_color=[6, 5, 4])
    tm = GbVmTensor('coarse_model', {'data_loader': {'ndc': False}, 'model': {'white_bkgd': False}}, tcfg,
                    {'bounding_box': bbox})
    tm.update_tensor_params(torch.tensor(g['res']), torch.tensor(g['bbox']))
    with torch.no_grad():
        for kind, plist in (('amask_planes_density', tm.matrices_density), ('amask_lines_density', tm.vectors_density),
                            ('planes_color', tm.matrices_color), ('lines_color', tm.vectors_color)):
            for i in range(3):
                plist[i] = torch.nn.Parameter(T.to_channels_last(torch.from_numpy(g[f'{kind}.{i}'])[None]))
    tm = tm.to(DEV)
    np.testing.assert_allclose(float(tm.step_size), float(g['amask_step_size']), rtol=1e-6)
    box = tm.update_alpha_mask(0).cpu().numpy()
    vol = tm.alpha_mask.volume().cpu().numpy()
    ref = g['amask_volume']
    assert vol.shape == ref.shape
    assert np.mean(vol != ref) <= 1e-3, np.mean(vol != ref)
    voxel = (g['bbox'][1] - g['bbox'][0]) / (g['res'] - 1)
    assert np.all(np.abs(box - g['amask_box']) <= voxel * 1.0001), (box, g['amask_box'])


@pytest.mark.parametrize('tag', ['ndc', 'world', 'synthetic'])
def test_drop_in_tensorf_forward_from_pixels_matches_reference(golden, tag):
    """GbSimpleTensoRF.forward from pixel ids against SimpleTensoRF.forward in
    evaluation mode (golden tensorf_e2e): rays with the half pixel and the x-flip,
    NDC rays and view directions, the NeRF-Synthetic convention, NDC / AABB
    marching, the coarse VM model, and the static-camera view directions of a
    separate view pose (SimpleTensoRF09.py:194-238, 353-401)."""
    from simple_rf_gb300.tensorf_model import GbSimpleTensoRF
    g = golden('tensorf_e2e')
    ndc = tag == 'ndc'
    bbox = [[-1.5, -1.67, -1.0], [1.5, 1.67, 1.0]] if ndc else [[-1.5] * 3, [1.5] * 3]
    cfg = dict(_tcfg(), bounding_box=bbox, num_components_density=[16, 4, 4], num_components_color=[48, 12, 12],
               num_voxels_initial=16 ** 3, num_voxels_final=16 ** 3, features_dimension_color=27,
               num_units_color_predictor=128)
    model = {'name': 'GbSimpleTensoRF01', 'coarse_model': cfg, 'learn_camera_focal_length': False,
             'learn_camera_rotation': False, 'learn_camera_translation': False, 'chunk': 1 << 16, 'lindisp': False,
             'perturb': True, 'white_bkgd': not ndc}
    mc = {'intrinsics': g['intrinsics'], 'extrinsics': g[f'{tag}_extrinsics'], 'resolution': (378, 504),
          'near': 1.0 if ndc else 2.0, 'far': 100.0 if ndc else 6.0, 'near_ndc': 0.0, 'far_ndc': 1.0,
          'bounding_box': np.array(bbox)}
    database = 'NeRF_Synthetic' if tag == 'synthetic' else 'NeRF_LLFF'
    m = GbSimpleTensoRF({'data_loader': {'ndc': ndc}, 'model': model, 'database': database}, mc)
    sd = {k[len(tag) + 4:]: torch.from_numpy(g[k]) for k in g if k.startswith(f'{tag}_sd.')}
    m.load_state_dict(sd)
    m = m.to(DEV).eval()
    pix = torch.from_numpy(g['pixel_id']).to(DEV)
    batch = {'pixel_id': pix, 'num_frames': 1, 'iter_num': 1, 'sub_batch_index': 1, 'common_data': {}}
    with torch.no_grad():
        ret = m(batch, retraw=True)
        sbatch = dict(batch, common_data={'view_intrinsic': None, 'processed_view_pose':
                                          torch.from_numpy(g['view_pose']).float()[None].to(DEV)})
        ret_s = m(sbatch, retraw=True, mode='static_camera')
    ref = {k[len(tag) + 5:]: g[k] for k in g if k.startswith(f'{tag}_out.')}
    got = {k: v.cpu().numpy() for k, v in ret.items() if isinstance(v, torch.Tensor)}
    assert set(ref) <= set(got), set(ref) - set(got)
    keep = threshold_stable(got['weights_coarse'], ref['weights_coarse'])
    assert keep.sum() >= keep.size - 1, int((~keep).sum())
    for k in ('rays_o', 'rays_d', 'view_dirs', 'z_vals_coarse') + (('rays_o_ndc', 'rays_d_ndc') if ndc else ()):
        np.testing.assert_allclose(got[k], ref[k], rtol=1e-5, atol=1e-6 * max(1.0, float(np.abs(ref[k]).max())),
                                   err_msg=k)
    for k in ('rgb_coarse', 'depth_coarse', 'acc_coarse', 'weights_coarse', 'depth_var_coarse') + \
            (('depth_ndc_coarse',) if ndc else ()):
        np.testing.assert_allclose(got[k][keep], ref[k][keep], rtol=1e-5,
                                   atol=1e-6 * max(1.0, float(np.abs(ref[k]).max())), err_msg=k)
    for k in ('view_dirs', 'rgb_coarse', 'depth_coarse'):
        r = g[f'{tag}_static.{k}']
        np.testing.assert_allclose(ret_s[k].cpu().numpy()[keep], r[keep], rtol=1e-5,
                                   atol=1e-6 * max(1.0, float(np.abs(r).max())), err_msg='static ' + k)


@pytest.mark.parametrize('precision', ['fp16', 'bf16'])
def test_basis_adjoint_tensor_cores_match_simt(precision):
    """The 16-bit renderer backward's two basis adjoints on the same inputs: the TF32
    tensor-core pass (d_feats = dB . Wb) with its dWb reduction against the fused
    FP32 SIMT pass.  d_feats and dWb within 3e-3 relative L2 (TF32 keeps 10 mantissa
    bits of dB and Wb); every other gradient is the same computation (1e-5)."""
    from simple_rf_gb300 import _lib, build as b, tensorf as T
    b.build()
    from simple_rf_gb300.bench_tensorf import make_models
    tm = make_models(DEV, seed=4, precision=precision, grids=(64, 32))[0]
    cp = tm.color_predictor
    gen = torch.Generator(device=DEV).manual_seed(8)
    m = 20000 + 37
    feats = torch.randn(m, 144, device=DEV, generator=gen) * 0.3
    vd = torch.nn.functional.normalize(torch.randn(m, 3, device=DEV, generator=gen), dim=-1)
    g_rgb = torch.rand(m, 3, device=DEV, generator=gen) * 1e-3
    desc = _lib.RendererDesc(144, cp.features_dimension, cp.mlp[0].out_features, cp.lf, cp.lv, 1)
    params = [tm.basis_matrix_color.weight, cp.mlp[0].weight, cp.mlp[0].bias, cp.mlp[2].weight, cp.mlp[2].bias,
              cp.mlp[4].weight, cp.mlp[4].bias]
    prec = _lib.PRECISIONS[precision]
    res = {}
    lib = _lib.load()
    try:
        for path in (1, 0):
            _lib.check(lib.srf_tensorf_basis_adjoint_path(path), 'srf_tensorf_basis_adjoint_path')
            f = feats.clone().requires_grad_(True)
            ps = [p.detach().clone().requires_grad_(True) for p in params]
            T.renderer_tc(desc, prec, f, vd, ps).backward(g_rgb)
            torch.cuda.synchronize()
            res[path] = [f.grad] + [p.grad for p in ps]
    finally:
        lib.srf_tensorf_basis_adjoint_path(1)
    names = ['d_feats', 'basis', 'w1', 'b1', 'w2', 'b2', 'w3', 'b3']
    for name, tc_g, simt_g in zip(names, res[1], res[0]):
        rel = ((tc_g - simt_g).norm() / simt_g.norm()).item()
        print(precision, name, 'tensor-core vs SIMT adjoint rel-L2', rel)
        assert rel < (3e-3 if name in ('d_feats', 'basis') else 1e-5), (name, rel)
