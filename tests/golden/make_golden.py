"""Generate golden fixtures by running the reference Simple-RF model code on CPU.

Run in a container where the reference project is available (default
``/root/reference``; override with ``SRF_REFERENCE_ROOT``):

    python tests/golden/make_golden.py

The reference is imported read-only (``sys.dont_write_bytecode``) with a stub
for ``matplotlib`` (imported but unused by ``utils/CommonUtils04.py``).  Random
draws inside the reference (``torch.rand`` at SimpleNeRF17.py:355/397 and
SimpleTensoRF09.py:398) are replaced by explicit uniforms so every fixture is a
pure function of its stored inputs.  Weights come from numpy PCG64 seeds
(``oracle.nerf.xavier_params``) so the fixtures need not store them.
"""
import os
import sys
import types
import contextlib

import numpy as np
import torch

sys.dont_write_bytecode = True
REF = os.environ.get('SRF_REFERENCE_ROOT', '/root/reference')
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REF, 'src'))
sys.path.insert(0, REPO)
for name in ('matplotlib', 'matplotlib.pyplot'):
    sys.modules.setdefault(name, types.ModuleType(name))

from models import SimpleNeRF17 as RN  # noqa: E402
from models import SimpleTensoRF09 as RT  # noqa: E402
from utils import CommonUtils04 as CU  # noqa: E402
from oracle import nerf as onerf  # noqa: E402

torch.set_num_threads(4)


@contextlib.contextmanager
def patched_rand(queue):
    """Replace torch.rand / torch.rand_like by a queue of prepared tensors."""
    orig_rand, orig_like = torch.rand, torch.rand_like

    def fake(*args, **kwargs):
        t = queue.pop(0)
        return t.clone()

    torch.rand = fake
    torch.rand_like = fake
    try:
        yield
    finally:
        torch.rand, torch.rand_like = orig_rand, orig_like


def mlp_cfg(width=256, depth=8, wv=128, lp=10, lv=4, views=True, vdr=True, lps=None, ns=64):
    c = {'num_samples': ns, 'points_net_depth': depth, 'views_net_depth': 1, 'points_net_width': width,
         'views_net_width': wv, 'points_positional_encoding_degree': lp, 'views_positional_encoding_degree': lv,
         'use_view_dirs': views, 'view_dependent_rgb': vdr, 'predict_visibility': False}
    if lps is not None:
        c['points_sigma_positional_encoding_degree'] = lps
    return c


def nerf_configs(coarse, fine, ndc=False, white=False, augs=None):
    model = {'name': 'SimpleNeRF17', 'coarse_model': coarse, 'learn_camera_focal_length': False,
             'learn_camera_rotation': False, 'learn_camera_translation': False, 'chunk': 1 << 20,
             'lindisp': False, 'netchunk': 1 << 20, 'perturb': True, 'raw_noise_std': 0.0, 'white_bkgd': white}
    if fine is not None:
        model['fine_model'] = fine
    if augs:
        model['augmentations'] = augs
    configs = {'data_loader': {'ndc': ndc}, 'model': model, 'database': 'synthetic'}
    model_configs = {'intrinsics': np.eye(3)[None].repeat(1, 0), 'extrinsics': np.eye(4)[None].repeat(1, 0),
                     'resolution': (378, 504), 'near': 2.0 if not ndc else 1.0, 'far': 6.0,
                     'near_ndc': 0.0, 'far_ndc': 1.0}
    return configs, model_configs


def load_mlp(mlp, seed):
    spec = onerf.MlpSpec.from_config(mlp.mlp_configs)
    p = onerf.xavier_params(spec, seed)
    sd = {k: torch.from_numpy(v) for k, v in p.items()}
    missing = mlp.load_state_dict(sd, strict=True)
    assert not missing.missing_keys
    return spec, p


def synthetic_rays(n, seed):
    g = torch.Generator().manual_seed(seed)
    o = torch.randn(n, 3, generator=g) * 0.1
    d = torch.randn(n, 3, generator=g)
    d = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    return o, d


def ndc_world_rays(n, seed):
    """Forward-facing rays: origins on z=-1 with x,y ~ U[-1,1]; directions with z in [-1.2,-0.8]."""
    g = torch.Generator().manual_seed(seed)
    o = torch.empty(n, 3)
    o[:, :2] = torch.rand(n, 2, generator=g) * 2 - 1
    o[:, 2] = -1.0
    d = torch.empty(n, 3)
    d[:, :2] = torch.rand(n, 2, generator=g) * 0.4 - 0.2
    d[:, 2] = -(torch.rand(n, generator=g) * 0.4 + 0.8)
    d = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    return o, d


def render_case(n, sc, sf, seed, coarse_cfg, fine_cfg, ndc=False, white=False, augs=None, aug_seeds=None,
                with_grads=False):
    configs, model_configs = nerf_configs(coarse_cfg, fine_cfg, ndc=ndc, white=white, augs=augs)
    model = RN.SimpleNeRF(configs, model_configs)
    model.train()
    spec_c, pc = load_mlp(model.coarse_model, seed)
    spec_f, pf = load_mlp(model.fine_model, seed + 1)
    aug_seeds = aug_seeds or []
    for am, s in zip(getattr(model, 'augmented_models', []), aug_seeds):
        load_mlp(am['coarse_model'], s)
    rays_o, rays_d = ndc_world_rays(n, seed) if ndc else synthetic_rays(n, seed)
    g = torch.Generator().manual_seed(seed + 100)
    u_c = torch.rand(n, sc, generator=g)
    u_f = torch.rand(n, sf, generator=g)
    focal = 400.0
    intr = torch.tensor([[focal, 0, 252.0], [0, focal, 189.0], [0, 0, 1.0]])[None].repeat(n, 1, 1)
    inp = {'pixel_id': torch.zeros(n, 3, dtype=torch.int32), 'intrinsics': intr,
           'extrinsics': torch.eye(4)[None].repeat(n, 1, 1), 'common_data': {}, 'num_frames': 1}
    orig = RN.CommonUtils.get_rays_tr
    RN.CommonUtils.get_rays_tr = lambda *a, **k: (rays_o.clone(), rays_d.clone())
    try:
        with patched_rand([u_c, u_f]):
            ret = model.render_rays(inp, retraw=True, sec_views_vis=False, mode=None)
    finally:
        RN.CommonUtils.get_rays_tr = orig
    out = {'rays_o': rays_o.numpy(), 'rays_d': rays_d.numpy(), 'u_coarse': u_c.numpy(), 'u_fine': u_f.numpy(),
           'seed': np.array(seed), 'focal': np.array(focal)}
    for k, v in ret.items():
        out['out_' + k] = v.detach().numpy()
    if with_grads:
        tg = torch.Generator().manual_seed(seed + 200)
        t_rgb = torch.rand(n, 3, generator=tg)
        t_depth = torch.rand(n, generator=tg) * 4 + 2
        dmask = torch.zeros(n)
        dmask[:max(n // 4, 1)] = 1
        loss = 0
        for tag in ('coarse', 'fine'):
            loss = loss + torch.mean(torch.mean((ret[f'rgb_{tag}'] - t_rgb) ** 2, 1))
            loss = loss + 0.1 * torch.sum(torch.abs(ret[f'depth_{tag}'] - t_depth) * dmask) / dmask.sum()
        loss.backward()
        out['t_rgb'], out['t_depth'], out['dmask'] = t_rgb.numpy(), t_depth.numpy(), dmask.numpy()
        out['loss'] = np.array(loss.item())
        for tag, mlp in (('coarse', model.coarse_model), ('fine', model.fine_model)):
            for k, prm in mlp.named_parameters():
                out[f'grad_{tag}.{k}'] = prm.grad.numpy().copy()
    return out


def sampling_case():
    g = torch.Generator().manual_seed(7)
    n, sc, sf = 32, 64, 128
    u_c = torch.rand(n, sc, generator=g)
    fake = types.SimpleNamespace(ndc=False, training=True,
                                 configs={'model': {'perturb': True, 'lindisp': False,
                                                    'coarse_model': {'num_samples': sc},
                                                    'fine_model': {'num_samples': sf}}},
                                 model_configs={'near': 2.0, 'far': 6.0, 'near_ndc': 0.0, 'far_ndc': 1.0},
                                 sample_pdf=RN.SimpleNeRF.sample_pdf)
    inp = {'pixel_id': torch.zeros(n, 3)}
    with patched_rand([u_c]):
        zc = RN.SimpleNeRF.get_z_vals_coarse(fake, inp)
    fake.training = False
    zc_det = RN.SimpleNeRF.get_z_vals_coarse(fake, inp)
    w = torch.rand(n, sc, generator=g) ** 4
    w[0] = 0.0                      # all-zero weights: uniform pdf (+1e-5 floor)
    w[1, :] = 0.0
    w[1, 30] = 5.0                  # one spike
    w[2, ::2] = 0.0                 # alternating zeros -> denom < 1e-5 cases
    u_f = torch.rand(n, sf, generator=g)
    u_f[3, :4] = torch.tensor([0.0, 1.0, 0.5, 0.999999])
    fake.training = True
    with patched_rand([u_f]):
        zf = RN.SimpleNeRF.get_z_vals_fine(fake, zc, w)
    mids = .5 * (zc[..., 1:] + zc[..., :-1])
    with patched_rand([u_f]):
        samples = RN.SimpleNeRF.sample_pdf(mids, w[..., 1:-1], sf, det=False)
    samples_det = RN.SimpleNeRF.sample_pdf(mids, w[..., 1:-1], sf, det=True)
    fake.training = False
    zf_det = RN.SimpleNeRF.get_z_vals_fine(fake, zc, w)
    return {'u_coarse': u_c.numpy(), 'z_coarse': zc.numpy(), 'z_coarse_det': zc_det.numpy(), 'weights': w.numpy(),
            'u_fine': u_f.numpy(), 'z_fine': zf.numpy(), 'samples': samples.numpy(),
            'samples_det': samples_det.numpy(), 'z_fine_det': zf_det.numpy()}


def pe_case():
    g = torch.Generator().manual_seed(11)
    x = torch.randn(257, 3, generator=g) * 3
    x[0] = torch.tensor([0.0, -1.5, 1e-3])
    x[1] = torch.tensor([30.0, -41.0, 7.25])
    out = {'x': x.numpy()}
    for deg in (10, 4, 3, 2, 0):
        fn, dim = RN.MLP.get_positional_encoder(deg)
        out[f'pe{deg}'] = fn(x).numpy()
    return out


def mlp_case():
    g = torch.Generator().manual_seed(13)
    m = 96
    pts = torch.randn(m, 3, generator=g)
    vd = torch.randn(m, 3, generator=g)
    vd = vd / torch.linalg.norm(vd, dim=-1, keepdim=True)
    out = {'pts': pts.numpy(), 'vdirs': vd.numpy()}
    variants = {
        'main': mlp_cfg(),
        'aug_l4_noview': mlp_cfg(lp=4, views=False, vdr=False),
        'points_aug': mlp_cfg(lps=3),
    }
    configs, _ = nerf_configs(mlp_cfg(), None)
    for i, (name, cfg) in enumerate(variants.items()):
        mlp = RN.MLP(name, configs, cfg, {})
        mlp.eval()
        load_mlp(mlp, 1000 + i)
        res = mlp({'pts': pts, 'view_dirs': vd})
        out[f'{name}_sigma'] = res['sigma'].detach().numpy()
        out[f'{name}_rgb'] = res['rgb'].detach().numpy()
    return out


def composite_case():
    out = {}
    g = torch.Generator().manual_seed(17)
    n, s = 24, 48
    for ndc in (False, True):
        tag = 'ndc' if ndc else 'world'
        configs, _ = nerf_configs(mlp_cfg(), None, ndc=ndc, white=True)
        fake = types.SimpleNamespace(ndc=ndc, configs=configs, predict_visibility=False,
                                     convert_depth_from_ndc=RN.SimpleNeRF.convert_depth_from_ndc)
        sigma = (torch.randn(n, s, 1, generator=g) * 2).relu()
        sigma[0] = 0.0
        sigma[1, 5:] = 1e4
        rgb = torch.rand(n, s, 3, generator=g)
        if ndc:
            o, d = ndc_world_rays(n, 3)
            intr = torch.tensor([[400.0, 0, 252.0], [0, 400.0, 189.0], [0, 0, 1.0]])[None].repeat(n, 1, 1)
            o_ndc, d_ndc = CU.get_ndc_rays_tr(o, d, (378, 504), intr, near=1.0)
            z = torch.sort(torch.rand(n, s, generator=g), -1)[0]
            z[2, -1] = 1.0
        else:
            o, d = synthetic_rays(n, 4)
            d = d * (1 + torch.rand(n, 1, generator=g))
            z = 2 + 4 * torch.sort(torch.rand(n, s, generator=g), -1)[0]
            o_ndc = d_ndc = None
        sigma.requires_grad_(True)
        rgb.requires_grad_(True)
        if ndc:
            res = RN.SimpleNeRF.volume_rendering(fake, {'sigma': sigma, 'rgb': rgb}, z_vals_ndc=z, rays_d_ndc=d_ndc,
                                                 rays_o=o, rays_d=d)
        else:
            res = RN.SimpleNeRF.volume_rendering(fake, {'sigma': sigma, 'rgb': rgb}, z_vals=z, rays_d=d)
        gw = torch.Generator().manual_seed(19)
        loss = 0
        for k in sorted(res):
            c = torch.randn(res[k].shape, generator=gw)
            out[f'{tag}_cot_{k}'] = c.numpy()
            loss = loss + torch.sum(res[k] * c) if k not in ('alpha', 'visibility') else loss
            out[f'{tag}_out_{k}'] = res[k].detach().numpy()
        loss.backward()
        out[f'{tag}_sigma'] = sigma.detach().numpy()[..., 0]
        out[f'{tag}_rgb'] = rgb.detach().numpy()
        out[f'{tag}_z'] = z.numpy()
        out[f'{tag}_rays_o'] = o.numpy()
        out[f'{tag}_rays_d'] = d.numpy()
        if ndc:
            out[f'{tag}_rays_d_ndc'] = d_ndc.numpy()
            out[f'{tag}_rays_o_ndc'] = o_ndc.numpy()
        out[f'{tag}_dsigma'] = sigma.grad.numpy()[..., 0]
        out[f'{tag}_drgb'] = rgb.grad.numpy()
    return out


def rays_case():
    g = torch.Generator().manual_seed(23)
    n = 40
    pix = torch.stack([torch.zeros(n, dtype=torch.int64), torch.randint(0, 504, (n,), generator=g),
                       torch.randint(0, 378, (n,), generator=g)], 1).int()
    intr = torch.tensor([[400.0, 0, 252.0], [0, 400.0, 189.0], [0, 0, 1.0]])[None].repeat(n, 1, 1)
    ext = torch.eye(4)[None].repeat(n, 1, 1)
    ext[:, :3, 3] = torch.rand(n, 3, generator=g) * 0.2 - 0.1
    o, d = CU.get_rays_tr(pix, intr, ext, mip_nerf_used=False)
    o2, d2 = CU.get_rays_tr(pix, intr, ext, mip_nerf_used=True)
    on, dn = CU.get_ndc_rays_tr(o, d, (378, 504), intr, near=1.0)
    vd = CU.get_view_dirs_tr(d)
    return {'pixel_id': pix.numpy(), 'intrinsics': intr.numpy(), 'extrinsics': ext.numpy(), 'rays_o': o.numpy(),
            'rays_d': d.numpy(), 'rays_o_half': o2.numpy(), 'rays_d_half': d2.numpy(), 'rays_o_ndc': on.numpy(),
            'rays_d_ndc': dn.numpy(), 'view_dirs': vd.numpy()}


def tensorf_case():
    """VM density/colour, alpha mask, renderer MLP and LowRankTensor.forward on a small grid."""
    g = torch.Generator().manual_seed(29)
    res = torch.tensor([20, 22, 24])
    bbox = [[-1.5, -1.5, -1.5], [1.5, 1.5, 1.5]]
    tcfg = {'decomposition_type': 'VectorMatrix', 'num_samples_max': 1e6, 'num_components_density': [4, 3, 2],
            'num_components_color': [6, 5, 4], 'bounding_box': bbox, 'num_voxels_initial': int(res.prod()),
            'num_voxels_final': int(res.prod()), 'tensor_upsampling_iters': [], 'num_voxels_per_sample': 0.5,
            'alpha_mask_update_iters': [], 'alpha_mask_threshold': 1e-4, 'ray_marching_weight_threshold': 1e-4,
            'use_view_dirs': True, 'view_dependent_color': True, 'views_positional_encoding_degree': 2,
            'features_positional_encoding_degree': 2, 'features_dimension_color': 7, 'density_offset': -10,
            'distance_scale': 25, 'density_predictor': 'ReLU', 'color_predictor': 'MLP_Features',
            'num_units_color_predictor': 16, 'predict_visibility': False}
    configs = {'data_loader': {'ndc': False}, 'model': {'white_bkgd': False}, 'database': 'synthetic'}
    tm = RT.VmDecomposedTensor('coarse_model', configs, tcfg, {'bounding_box': bbox})
    tm.update_tensor_params(res, torch.tensor(bbox))
    tm.matrices_density, tm.vectors_density = tm.create_decomposed_tensor([4, 3, 2], res, 0.1)
    tm.matrices_color, tm.vectors_color = tm.create_decomposed_tensor([6, 5, 4], res, 0.1)
    with torch.no_grad():
        for plist in (tm.matrices_density, tm.vectors_density):
            for prm in plist:
                prm.copy_(torch.randn(prm.shape, generator=g) * 0.3 + 0.15)
        for plist in (tm.matrices_color, tm.vectors_color):
            for prm in plist:
                prm.copy_(torch.randn(prm.shape, generator=g) * 0.3)
        for prm in list(tm.basis_matrix_color.parameters()) + list(tm.color_predictor.parameters()):
            prm.copy_(torch.randn(prm.shape, generator=g) * 0.3)
    vol = (torch.rand(12, 10, 8, generator=g) < 0.3).float()
    tm.alpha_mask = RT.AlphaGridMask(vol, torch.tensor(bbox))
    tm.train()
    n = 12
    o = torch.zeros(n, 3)
    o[:, 2] = -3.0
    o[:, :2] = torch.rand(n, 2, generator=g) * 0.6 - 0.3
    d = torch.randn(n, 3, generator=g) * 0.15
    d[:, 2] = 1.0
    d = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    u = torch.rand(n, 1, generator=g)
    fake = types.SimpleNamespace(ndc=False, training=True,
                                 configs={'model': {'perturb': True, 'lindisp': False}},
                                 model_configs={'near': 0.5, 'far': 6.0})
    with patched_rand([u]):
        z = RT.SimpleTensoRF.get_z_vals_coarse(fake, {'pixel_id': torch.zeros(n, 3)},
                                               {'rays_o': o, 'rays_d': d}, tm)
    pts = o[:, None, :] + d[:, None, :] * z[:, :, None]
    vdir = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    inp = {'pts': pts, 'z_vals': z, 'rays_o': o, 'rays_d': d, 'view_dirs': vdir}
    with patched_rand([torch.tensor([0.25])]):       # white-background coin: rand < 0.5 -> white
        ret = tm(inp, retraw=True)
    tg = torch.Generator().manual_seed(31)
    loss = 0
    out = {}
    for k in ('rgb', 'depth', 'acc'):
        c = torch.randn(ret[k].shape, generator=tg)
        out[f'cot_{k}'] = c.numpy()
        loss = loss + torch.sum(ret[k] * c)
    loss.backward()
    out.update({'res': res.numpy(), 'bbox': np.array(bbox, np.float32), 'alpha_vol': vol.numpy(), 'u': u.numpy(),
                'rays_o': o.numpy(), 'rays_d': d.numpy(), 'z': z.numpy(), 'step_size': tm.step_size.numpy(),
                'num_samples': tm.num_samples.numpy()})
    for i in range(3):
        out[f'planes_density.{i}'] = tm.matrices_density[i].detach().numpy()[0]
        out[f'lines_density.{i}'] = tm.vectors_density[i].detach().numpy()[0]
        out[f'planes_color.{i}'] = tm.matrices_color[i].detach().numpy()[0]
        out[f'lines_color.{i}'] = tm.vectors_color[i].detach().numpy()[0]
        out[f'grad_planes_density.{i}'] = tm.matrices_density[i].grad.numpy()[0]
        out[f'grad_lines_density.{i}'] = tm.vectors_density[i].grad.numpy()[0]
        out[f'grad_planes_color.{i}'] = tm.matrices_color[i].grad.numpy()[0]
        out[f'grad_lines_color.{i}'] = tm.vectors_color[i].grad.numpy()[0]
    out['basis_matrix_color.weight'] = tm.basis_matrix_color.weight.detach().numpy()
    out['grad_basis_matrix_color.weight'] = tm.basis_matrix_color.weight.grad.numpy()
    for k, prm in tm.color_predictor.named_parameters():
        out['color_predictor.' + k] = prm.detach().numpy()
        out['grad_color_predictor.' + k] = prm.grad.numpy()
    for k, v in ret.items():
        out['out_' + k] = v.detach().numpy()
    # alpha-mask query alone, including points on grid nodes / faces and outside the box
    q = torch.rand(300, 3, generator=g) * 3.4 - 1.7
    q[:8] = torch.tensor([[-1.5, -1.5, -1.5], [1.5, 1.5, 1.5], [0.0, 0.0, 0.0], [-1.5, 0.3, 1.5],
                          [1.5000001, 0, 0], [0.1, -1.5, 0.2], [-1.0714285, 0.5, -0.4285714], [0.5, 0.5, 0.5]])
    out['alpha_q'] = q.numpy()
    out['alpha_q_pos'] = (tm.alpha_mask.sample_alpha(q) > 0).numpy()
    return out


def tensorf_ndc_case():
    """LowRankTensor.forward in NDC mode (the reference's forward-facing TensoRF
    configuration, NerfLlffTrainerTester10.py:894-1087: NDC bounding box, stratified
    NDC depths from get_z_vals_coarse :364-381, NDC marching points, metric depth via
    CommonUtils04.convert_depth_from_ndc) on a small grid, with autograd gradients."""
    g = torch.Generator().manual_seed(41)
    res = torch.tensor([20, 22, 24])
    bbox = [[-1.5, -1.67, -1.0], [1.5, 1.67, 1.0]]
    tcfg = {'decomposition_type': 'VectorMatrix', 'num_samples_max': 1e6, 'num_components_density': [4, 3, 2],
            'num_components_color': [6, 5, 4], 'bounding_box': bbox, 'num_voxels_initial': int(res.prod()),
            'num_voxels_final': int(res.prod()), 'tensor_upsampling_iters': [], 'num_voxels_per_sample': 0.5,
            'alpha_mask_update_iters': [], 'alpha_mask_threshold': 1e-4, 'ray_marching_weight_threshold': 1e-4,
            'use_view_dirs': True, 'view_dependent_color': True, 'views_positional_encoding_degree': 2,
            'features_positional_encoding_degree': 2, 'features_dimension_color': 7, 'density_offset': -10,
            'distance_scale': 25, 'density_predictor': 'ReLU', 'color_predictor': 'MLP_Features',
            'num_units_color_predictor': 16, 'predict_visibility': False}
    configs = {'data_loader': {'ndc': True}, 'model': {'white_bkgd': False}, 'database': 'synthetic'}
    tm = RT.VmDecomposedTensor('coarse_model', configs, tcfg, {'bounding_box': bbox})
    tm.update_tensor_params(res, torch.tensor(bbox))
    tm.matrices_density, tm.vectors_density = tm.create_decomposed_tensor([4, 3, 2], res, 0.1)
    tm.matrices_color, tm.vectors_color = tm.create_decomposed_tensor([6, 5, 4], res, 0.1)
    with torch.no_grad():
        for plist in (tm.matrices_density, tm.vectors_density):
            for prm in plist:
                prm.copy_(torch.randn(prm.shape, generator=g) * 0.3 + 0.15)
        for plist in (tm.matrices_color, tm.vectors_color):
            for prm in plist:
                prm.copy_(torch.randn(prm.shape, generator=g) * 0.3)
        for prm in list(tm.basis_matrix_color.parameters()) + list(tm.color_predictor.parameters()):
            prm.copy_(torch.randn(prm.shape, generator=g) * 0.3)
    vol = (torch.rand(12, 10, 8, generator=g) < 0.3).float()
    tm.alpha_mask = RT.AlphaGridMask(vol, torch.tensor(bbox))
    tm.train()
    n = 12
    o, d = ndc_world_rays(n, 43)
    intr = torch.tensor([[400.0, 0, 252.0], [0, 400.0, 189.0], [0, 0, 1.0]])[None].repeat(n, 1, 1)
    o_ndc, d_ndc = CU.get_ndc_rays_tr(o, d, (378, 504), intr, near=1.0)
    s = int(tm.num_samples.item())
    u = torch.rand(n, s, generator=g)
    fake = types.SimpleNamespace(ndc=True, training=True,
                                 configs={'model': {'perturb': True, 'lindisp': False}},
                                 model_configs={'near': 1.0, 'far': 100.0, 'near_ndc': 0.0, 'far_ndc': 1.0})
    with patched_rand([u]):
        z = RT.SimpleTensoRF.get_z_vals_coarse(fake, {'pixel_id': torch.zeros(n, 3)}, {'rays_o': o, 'rays_d': d}, tm)
    pts = o_ndc[:, None, :] + d_ndc[:, None, :] * z[:, :, None]
    vdir = CU.get_view_dirs_tr(d_ndc)
    inp = {'pts': pts, 'z_vals': z, 'z_vals_ndc': z, 'rays_o': o, 'rays_d': d, 'rays_d_ndc': d_ndc,
           'view_dirs': vdir}
    with patched_rand([torch.tensor([0.75])]):       # white-background coin: rand >= 0.5 -> no white
        ret = tm(inp, retraw=True)
    tg = torch.Generator().manual_seed(47)
    loss = 0
    out = {}
    for k in ('rgb', 'depth', 'depth_ndc', 'acc'):
        c = torch.randn(ret[k].shape, generator=tg)
        out[f'cot_{k}'] = c.numpy()
        loss = loss + torch.sum(ret[k] * c)
    loss.backward()
    out.update({'res': res.numpy(), 'bbox': np.array(bbox, np.float32), 'alpha_vol': vol.numpy(), 'u': u.numpy(),
                'rays_o': o.numpy(), 'rays_d': d.numpy(), 'rays_o_ndc': o_ndc.numpy(), 'rays_d_ndc': d_ndc.numpy(),
                'view_dirs': vdir.numpy(), 'z': z.numpy(), 'num_samples': tm.num_samples.numpy()})
    for i in range(3):
        out[f'planes_density.{i}'] = tm.matrices_density[i].detach().numpy()[0]
        out[f'lines_density.{i}'] = tm.vectors_density[i].detach().numpy()[0]
        out[f'planes_color.{i}'] = tm.matrices_color[i].detach().numpy()[0]
        out[f'lines_color.{i}'] = tm.vectors_color[i].detach().numpy()[0]
        out[f'grad_planes_density.{i}'] = tm.matrices_density[i].grad.numpy()[0]
        out[f'grad_lines_density.{i}'] = tm.vectors_density[i].grad.numpy()[0]
        out[f'grad_planes_color.{i}'] = tm.matrices_color[i].grad.numpy()[0]
        out[f'grad_lines_color.{i}'] = tm.vectors_color[i].grad.numpy()[0]
    out['basis_matrix_color.weight'] = tm.basis_matrix_color.weight.detach().numpy()
    out['grad_basis_matrix_color.weight'] = tm.basis_matrix_color.weight.grad.numpy()
    for k, prm in tm.color_predictor.named_parameters():
        out['color_predictor.' + k] = prm.detach().numpy()
        out['grad_color_predictor.' + k] = prm.grad.numpy()
    for k, v in ret.items():
        out['out_' + k] = v.detach().numpy()
    return out


REALISTIC = dict(seed=53, res=48, density=[16, 16, 16], color=[48, 48, 48], features=27, units=128, rays=256,
                 mask_res=32, mask_occupancy=0.15)


def tensorf_realistic_case():
    """LowRankTensor.forward at the benchmark's model shape on a 48^3 grid:
    16 / 48 components per plane and line, 27 features, 128 renderer units, PE
    L=2 on features and view directions, ReLU density, distance scale 25, a 32^3
    alpha mask at 15% occupancy, 256 rays marching from the sphere of radius 4
    (near 2, far 6) with one uniform per ray.  The parameters come from
    oracle.tensorf.seeded_vm_model and are not stored; the fixture holds the
    inputs, the outputs and the autograd gradients of a random-cotangent loss."""
    from oracle import tensorf as otf
    c = REALISTIC
    res = torch.tensor([c['res']] * 3)
    bbox = [[-1.5] * 3, [1.5] * 3]
    tcfg = dict(tensorf_cfg(int(res.prod()), c['density'], c['color'], bbox), views_positional_encoding_degree=2,
                features_positional_encoding_degree=2)
    configs = {'data_loader': {'ndc': False}, 'model': {'white_bkgd': True}, 'database': 'synthetic'}
    tm = RT.VmDecomposedTensor('coarse_model', configs, tcfg, {'bounding_box': bbox})
    tm.update_tensor_params(res, torch.tensor(bbox))
    assert [int(r) for r in tm.resolution] == [c['res']] * 3
    tp, _ = otf.seeded_vm_model(c['seed'], [c['res']] * 3, c['density'], c['color'], c['features'], c['units'])
    with torch.no_grad():
        for kind, mats, vecs in (('density', tm.matrices_density, tm.vectors_density),
                                 ('color', tm.matrices_color, tm.vectors_color)):
            for i in range(3):
                mats[i].copy_(torch.from_numpy(tp[f'planes_{kind}'][i])[None])
                vecs[i].copy_(torch.from_numpy(tp[f'lines_{kind}'][i])[None])
        tm.basis_matrix_color.weight.copy_(torch.from_numpy(tp['basis_matrix_color.weight']))
        for k, prm in tm.color_predictor.named_parameters():
            prm.copy_(torch.from_numpy(tp['color_predictor.' + k]))
    rng = np.random.default_rng(c['seed'] + 1)
    vol = torch.from_numpy((rng.random((c['mask_res'],) * 3) < c['mask_occupancy']).astype(np.float32))
    tm.alpha_mask = RT.AlphaGridMask(vol, torch.tensor(bbox))
    tm.eval()
    n = c['rays']
    o = rng.standard_normal((n, 3)).astype(np.float32)
    o = 4.0 * o / np.linalg.norm(o, axis=-1, keepdims=True)
    d = -o / 4.0 + 0.3 * rng.standard_normal((n, 3)).astype(np.float32)
    d = (d / np.linalg.norm(d, axis=-1, keepdims=True)).astype(np.float32)
    o, d = torch.from_numpy(o), torch.from_numpy(d)
    u = torch.from_numpy(rng.random((n, 1), dtype=np.float32))
    fake = types.SimpleNamespace(ndc=False, training=True,
                                 configs={'model': {'perturb': True, 'lindisp': False}},
                                 model_configs={'near': 2.0, 'far': 6.0})
    with patched_rand([u]):
        z = RT.SimpleTensoRF.get_z_vals_coarse(fake, {'pixel_id': torch.zeros(n, 3)},
                                               {'rays_o': o, 'rays_d': d}, tm)
    pts = o[:, None, :] + d[:, None, :] * z[:, :, None]
    vdir = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    ret = tm({'pts': pts, 'z_vals': z, 'rays_o': o, 'rays_d': d, 'view_dirs': vdir}, retraw=True)
    tg = torch.Generator().manual_seed(59)
    loss = 0
    out = {}
    for k in ('rgb', 'depth', 'acc'):
        cot = torch.randn(ret[k].shape, generator=tg)
        out[f'cot_{k}'] = cot.numpy()
        loss = loss + torch.sum(ret[k] * cot)
    loss.backward()
    out.update({'bbox': np.array(bbox, np.float32), 'alpha_vol': vol.numpy().astype(np.uint8), 'u': u.numpy(),
                'rays_o': o.numpy(), 'rays_d': d.numpy(), 'z': z.numpy(), 'step_size': tm.step_size.numpy(),
                'num_samples': tm.num_samples.numpy()})
    for k, v in c.items():
        out[f'cfg_{k}'] = np.array(v)
    for i in range(3):
        out[f'grad_planes_density.{i}'] = tm.matrices_density[i].grad.numpy()[0]
        out[f'grad_lines_density.{i}'] = tm.vectors_density[i].grad.numpy()[0]
        out[f'grad_planes_color.{i}'] = tm.matrices_color[i].grad.numpy()[0]
        out[f'grad_lines_color.{i}'] = tm.vectors_color[i].grad.numpy()[0]
    out['grad_basis_matrix_color.weight'] = tm.basis_matrix_color.weight.grad.numpy()
    for k, prm in tm.color_predictor.named_parameters():
        out['grad_color_predictor.' + k] = prm.grad.numpy()
    for k in ('rgb', 'depth', 'acc', 'weights', 'depth_var', 'raw_sigma'):
        out['out_' + k] = ret[k].detach().numpy()
    return out


def _pose(angle, t):
    c, s = np.cos(angle), np.sin(angle)
    e = np.eye(4)
    e[:3, :3] = [[c, 0, s], [0, 1, 0], [-s, 0, c]]
    e[:3, 3] = t
    return e


def tensorf_e2e_case():
    """SimpleTensoRF.forward from pixel ids in evaluation mode: ray generation with
    the half pixel and the x-flip (SimpleTensoRF09.py:194-210), NDC rays and view
    directions (:211-238), NDC / AABB marching (:353-401), the coarse VM model, and
    the static-camera view directions of a separate view pose (:222-232); in NDC
    (NeRF-LLFF), world and NeRF-Synthetic conventions.  The state_dicts are stored
    so the drop-in loads the same weights."""
    torch.manual_seed(0)
    intr = np.array([[[400.0, 0, 252.0], [0, 400.0, 189.0], [0, 0, 1.0]]])
    view_pose = _pose(-0.05, [0.1, 0.0, 0.2])
    g = torch.Generator().manual_seed(61)
    n = 64
    pix = torch.stack([torch.zeros(n, dtype=torch.long), torch.randint(0, 504, (n,), generator=g),
                       torch.randint(0, 378, (n,), generator=g)], 1)
    out = {'pixel_id': pix.numpy(), 'intrinsics': intr, 'view_pose': view_pose}
    # forward-facing camera near the origin for NDC; outside the box, looking at it, otherwise
    cases = (('ndc', True, 'NeRF_LLFF', [[-1.5, -1.67, -1.0], [1.5, 1.67, 1.0]], 1.0, 100.0, [0.05, -0.02, 0.3]),
             ('world', False, 'NeRF_LLFF', [[-1.5] * 3, [1.5] * 3], 2.0, 6.0, [0.05, -0.02, 4.0]),
             ('synthetic', False, 'NeRF_Synthetic', [[-1.5] * 3, [1.5] * 3], 2.0, 6.0, [0.05, -0.02, 4.0]))
    for tag, ndc, database, bbox, near, far, t in cases:
        ext = _pose(0.1, t)[None]
        out[f'{tag}_extrinsics'] = ext
        cfg = dict(tensorf_cfg(16 ** 3, [16, 4, 4], [48, 12, 12], bbox), views_positional_encoding_degree=2,
                   features_positional_encoding_degree=2)
        model = {'name': 'SimpleTensoRF09', 'coarse_model': cfg, 'learn_camera_focal_length': False,
                 'learn_camera_rotation': False, 'learn_camera_translation': False, 'chunk': 1 << 16,
                 'lindisp': False, 'perturb': True, 'white_bkgd': not ndc}
        model_configs = {'intrinsics': intr, 'extrinsics': ext, 'resolution': (378, 504), 'near': near, 'far': far,
                         'near_ndc': 0.0, 'far_ndc': 1.0, 'bounding_box': np.array(bbox)}
        m = RT.SimpleTensoRF({'data_loader': {'ndc': ndc}, 'model': model, 'database': database}, model_configs)
        with torch.no_grad():
            for prm in m.coarse_model.matrices_density:
                prm.add_(0.2)
            for prm in m.coarse_model.vectors_density:
                prm.add_(0.2)
        m.eval()
        batch = {'pixel_id': pix, 'num_frames': 1, 'iter_num': 1, 'sub_batch_index': 1, 'common_data': {}}
        with torch.no_grad():
            ret = m(batch, retraw=True)
            sbatch = dict(batch, common_data={'view_intrinsic': None,
                                              'processed_view_pose': torch.from_numpy(view_pose).float()[None]})
            ret_s = m(sbatch, retraw=True, mode='static_camera')
        for k, v in m.state_dict().items():
            out[f'{tag}_sd.{k}'] = v.numpy()
        for k, v in ret.items():
            if isinstance(v, torch.Tensor):
                out[f'{tag}_out.{k}'] = v.numpy()
        for k in ('view_dirs', 'rgb_coarse', 'depth_coarse'):
            out[f'{tag}_static.{k}'] = ret_s[k].numpy()
        assert float(ret['acc_coarse'].max()) > 0.05, (tag, float(ret['acc_coarse'].max()))
    return out


def tensorf_cfg(vox, dens, col, bbox):
    return {'decomposition_type': 'VectorMatrix', 'num_samples_max': 1e6, 'num_components_density': dens,
            'num_components_color': col, 'bounding_box': bbox, 'num_voxels_initial': vox, 'num_voxels_final': vox,
            'tensor_upsampling_iters': [], 'num_voxels_per_sample': 0.5, 'alpha_mask_update_iters': [],
            'alpha_mask_threshold': 1e-4, 'ray_marching_weight_threshold': 1e-4, 'use_view_dirs': True,
            'view_dependent_color': True, 'views_positional_encoding_degree': 0,
            'features_positional_encoding_degree': 0, 'features_dimension_color': 27, 'density_offset': -10,
            'distance_scale': 25, 'density_predictor': 'ReLU', 'color_predictor': 'MLP_Features',
            'num_units_color_predictor': 128, 'predict_visibility': False}


def state_dict_case():
    """state_dict keys and shapes of the reference's SimpleNeRF (main coarse + fine
    nets, a views and a points augmentation, camera learners) and SimpleTensoRF
    (main VM model and an augmented one at NDC bounding box), the configurations
    of the reference's demos at reduced grid sizes; the drop-in models must
    produce the same so checkpoints load either way."""
    augs = [{'name': 'views_augmentation', 'coarse_model': mlp_cfg(lp=4, views=False, vdr=False)},
            {'name': 'points_augmentation', 'coarse_model': mlp_cfg(lps=3)}]
    configs, model_configs = nerf_configs(mlp_cfg(ns=64), mlp_cfg(ns=128), ndc=True, augs=augs)
    nerf = RN.SimpleNeRF(configs, model_configs)
    bbox = [[-1.5, -1.67, -1.0], [1.5, 1.67, 1.0]]
    model = {'name': 'SimpleTensoRF09', 'coarse_model': tensorf_cfg(24 ** 3, [16, 4, 4], [48, 12, 12], bbox),
             'augmentations': [{'name': 'points_augmentation',
                                'coarse_model': tensorf_cfg(12 ** 3, [16, 4, 4], [48, 12, 12], bbox)}],
             'learn_camera_focal_length': False, 'learn_camera_rotation': False, 'learn_camera_translation': False,
             'chunk': 1 << 16, 'lindisp': False, 'perturb': True, 'white_bkgd': False}
    tconfigs = {'data_loader': {'ndc': True}, 'model': model, 'database': 'NeRF_LLFF'}
    tmodel_configs = dict(model_configs, bounding_box=np.array(bbox))
    tensorf = RT.SimpleTensoRF(tconfigs, tmodel_configs)
    cp_cfg = dict(tensorf_cfg(24 ** 3, [16], [48], bbox), decomposition_type='CandecompParafac')
    cp_model = dict(model, coarse_model=cp_cfg)
    del cp_model['augmentations']
    tensorf_cp = RT.SimpleTensoRF(dict(tconfigs, model=cp_model), dict(model_configs, bounding_box=np.array(bbox)))
    out = {}
    opt = {'lr_initial': 5e-4, 'lr_initial_tensor': 0.02, 'lr_initial_network': 1e-3}
    for tag, m in (('nerf', nerf), ('tensorf', tensorf), ('tensorf_cp', tensorf_cp)):
        out[f'{tag}_keys'] = np.array([f"{k}:{'x'.join(str(d) for d in v.shape)}" for k, v in m.state_dict().items()])
        # the optimizer's parameter groups (Trainer10.py:509-520 reads them): name, lr, parameter shapes
        out[f'{tag}_groups'] = np.array([f"{g['name']}|{g['lr']}|" + ','.join('x'.join(str(d) for d in p.shape)
                                                                           for p in g['params'])
                                         for g in m.get_trainable_parameters(opt)])
    return out


def output_keys_case():
    """Keys and shapes of the reference models' forward output dicts, in training
    mode (augmented models run, raw outputs kept) and in evaluation mode, for
    the configurations of state_dict_case on 8 pixels of one frame: the contract
    Trainer10, Tester07 and the loss functions consume."""
    torch.manual_seed(0)
    augs = [{'name': 'views_augmentation', 'coarse_model': mlp_cfg(lp=4, views=False, vdr=False)},
            {'name': 'points_augmentation', 'coarse_model': mlp_cfg(lps=3)}]
    configs, model_configs = nerf_configs(mlp_cfg(ns=16), mlp_cfg(ns=32), ndc=True, augs=augs)
    model_configs['intrinsics'] = np.array([[[400.0, 0, 252.0], [0, 400.0, 189.0], [0, 0, 1.0]]])
    nerf = RN.SimpleNeRF(configs, model_configs)
    bbox = [[-1.5, -1.67, -1.0], [1.5, 1.67, 1.0]]
    model = {'name': 'SimpleTensoRF09', 'coarse_model': tensorf_cfg(24 ** 3, [16, 4, 4], [48, 12, 12], bbox),
             'augmentations': [{'name': 'points_augmentation',
                                'coarse_model': tensorf_cfg(12 ** 3, [16, 4, 4], [48, 12, 12], bbox)}],
             'learn_camera_focal_length': False, 'learn_camera_rotation': False, 'learn_camera_translation': False,
             'chunk': 1 << 16, 'lindisp': False, 'perturb': True, 'white_bkgd': False}
    tconfigs = {'data_loader': {'ndc': True}, 'model': model, 'database': 'NeRF_LLFF'}
    tensorf = RT.SimpleTensoRF(tconfigs, dict(model_configs, bounding_box=np.array(bbox)))
    g = torch.Generator().manual_seed(3)
    pix = torch.stack([torch.zeros(8, dtype=torch.long), torch.randint(0, 504, (8,), generator=g),
                       torch.randint(0, 378, (8,), generator=g)], 1)
    batch = {'pixel_id': pix, 'num_frames': 1, 'iter_num': 1, 'sub_batch_index': 1, 'common_data': {}}
    out = {}
    for tag, m in (('nerf', nerf), ('tensorf', tensorf)):
        for mode, train in (('train', True), ('eval', False)):
            m.train(train)
            with torch.set_grad_enabled(train):
                ret = m(batch, retraw=False)
            out[f'{tag}_{mode}'] = np.array(sorted(f"{k}:{'x'.join(str(d) for d in v.shape)}"
                                                   for k, v in ret.items() if isinstance(v, torch.Tensor)))
    out['pixel_id'] = pix.numpy()
    return out


def tensorf_maintenance_case():
    """VmDecomposedTensor's grid maintenance on a small grid: upsample_vectors_and_matrices
    to a new resolution (SimpleTensoRF09.py:1284-1301) and shrink_tensor to an occupied
    box (:899-914, 1303-1320, with an alpha mask of another resolution, so the box is
    snapped to the grid) -- the planes, lines, resolution, box and sample count after each."""
    g = torch.Generator().manual_seed(53)
    res = torch.tensor([20, 22, 24])
    bbox = [[-1.5, -1.5, -1.5], [1.5, 1.5, 1.5]]
    tcfg = {'decomposition_type': 'VectorMatrix', 'num_samples_max': 1e6, 'num_components_density': [4, 3, 2],
            'num_components_color': [6, 5, 4], 'bounding_box': bbox, 'num_voxels_initial': int(res.prod()),
            'num_voxels_final': int(res.prod()), 'tensor_upsampling_iters': [], 'num_voxels_per_sample': 0.5,
            'alpha_mask_update_iters': [], 'alpha_mask_threshold': 1e-4, 'ray_marching_weight_threshold': 1e-4,
            'use_view_dirs': True, 'view_dependent_color': True, 'views_positional_encoding_degree': 2,
            'features_positional_encoding_degree': 2, 'features_dimension_color': 7, 'density_offset': -10,
            'distance_scale': 25, 'density_predictor': 'ReLU', 'color_predictor': 'MLP_Features',
            'num_units_color_predictor': 16, 'predict_visibility': False}
    configs = {'data_loader': {'ndc': False}, 'model': {'white_bkgd': False}, 'database': 'synthetic'}
    tm = RT.VmDecomposedTensor('coarse_model', configs, tcfg, {'bounding_box': bbox})
    tm.update_tensor_params(res, torch.tensor(bbox))
    tm.matrices_density, tm.vectors_density = tm.create_decomposed_tensor([4, 3, 2], res, 0.1)
    tm.matrices_color, tm.vectors_color = tm.create_decomposed_tensor([6, 5, 4], res, 0.1)
    with torch.no_grad():
        for plist in (tm.matrices_density, tm.vectors_density, tm.matrices_color, tm.vectors_color):
            for prm in plist:
                prm.copy_(torch.randn(prm.shape, generator=g))
    out = {'res': res.numpy(), 'bbox': np.array(bbox, np.float32)}
    kinds = (('planes_density', 'matrices_density'), ('lines_density', 'vectors_density'),
             ('planes_color', 'matrices_color'), ('lines_color', 'vectors_color'))
    for kind, attr in kinds:
        for i in range(3):
            out[f'{kind}.{i}'] = getattr(tm, attr)[i].detach().numpy()[0].copy()
    res_up = torch.tensor([30, 28, 26])
    md, vd = tm.upsample_vectors_and_matrices(tm.matrices_density, tm.vectors_density, res_up)
    mcl, vcl = tm.upsample_vectors_and_matrices(tm.matrices_color, tm.vectors_color, res_up)
    out['res_up'] = res_up.numpy()
    for kind, plist in (('planes_density', md), ('lines_density', vd), ('planes_color', mcl), ('lines_color', vcl)):
        for i in range(3):
            out[f'up_{kind}.{i}'] = plist[i].detach().numpy()[0].copy()
    # the alpha-mask rebuild (:849-876) on a sparse density: planes shifted negative
    with torch.no_grad():
        dens0 = [(p.detach().clone(), l.detach().clone()) for p, l in zip(tm.matrices_density, tm.vectors_density)]
        for prm in tm.matrices_density:
            prm.mul_(0.3).sub_(0.25)
        for prm in tm.vectors_density:
            prm.mul_(0.3).add_(0.5)
        # confined to a window of the grid (3 voxels in from each face), so the
        # occupied box is smaller than the grid's
        for i in range(3):
            (a0, a1), v = tm.matrix_axes[i], tm.vector_axes[i]
            pm, lv = tm.matrices_density[i], tm.vectors_density[i]
            keep_p = torch.zeros_like(pm)
            keep_p[..., 3:int(res[a1]) - 4, 3:int(res[a0]) - 4] = 1
            keep_l = torch.zeros_like(lv)
            keep_l[..., 3:int(res[v]) - 4, :] = 1
            pm.mul_(keep_p)
            lv.mul_(keep_l)
    for i in range(3):
        out[f'amask_planes_density.{i}'] = tm.matrices_density[i].detach().numpy()[0].copy()
        out[f'amask_lines_density.{i}'] = tm.vectors_density[i].detach().numpy()[0].copy()
    box_alpha = tm.update_alpha_mask(0)
    out['amask_volume'] = tm.alpha_mask.alpha_volume.detach().numpy().reshape(tm.alpha_mask.alpha_volume.shape[-3:])
    out['amask_box'] = box_alpha.numpy()
    out['amask_step_size'] = tm.step_size.numpy()
    with torch.no_grad():
        for (p0, l0), pm, lv in zip(dens0, tm.matrices_density, tm.vectors_density):
            pm.copy_(p0)
            lv.copy_(l0)
    vol = (torch.rand(10, 12, 14, generator=g) < 0.3).float()
    tm.alpha_mask = RT.AlphaGridMask(vol, torch.tensor(bbox))
    box_new = torch.tensor([[-1.0, -1.2, -0.8], [1.1, 0.9, 1.3]])
    tm.shrink_tensor(box_new)
    out['alpha_vol'] = vol.numpy()
    out['box_new'] = box_new.numpy()
    for kind, attr in kinds:
        for i in range(3):
            out[f'shrunk_{kind}.{i}'] = getattr(tm, attr)[i].detach().numpy()[0].copy()
    out['shrunk_res'] = tm.resolution.numpy()
    out['shrunk_bbox'] = tm.bounding_box.numpy()
    out['shrunk_num_samples'] = tm.num_samples.numpy()
    out['shrunk_step_size'] = tm.step_size.numpy()
    return out


def tensorf_cp_case():
    """CP decomposition (CpDecomposedTensor, SimpleTensoRF09.py:964-1123): density and
    colour from three lines each, then the same renderer; LowRankTensor.forward on a
    small grid with autograd gradients."""
    g = torch.Generator().manual_seed(37)
    res = torch.tensor([18, 20, 22])
    bbox = [[-1.5, -1.5, -1.5], [1.5, 1.5, 1.5]]
    tcfg = {'decomposition_type': 'CandecompParafac', 'num_samples_max': 1e6, 'num_components_density': [5],
            'num_components_color': [6], 'bounding_box': bbox, 'num_voxels_initial': int(res.prod()),
            'num_voxels_final': int(res.prod()), 'tensor_upsampling_iters': [], 'num_voxels_per_sample': 0.5,
            'alpha_mask_update_iters': [], 'alpha_mask_threshold': 1e-4, 'ray_marching_weight_threshold': 1e-4,
            'use_view_dirs': True, 'view_dependent_color': True, 'views_positional_encoding_degree': 2,
            'features_positional_encoding_degree': 2, 'features_dimension_color': 7, 'density_offset': -10,
            'distance_scale': 25, 'density_predictor': 'ReLU', 'color_predictor': 'MLP_Features',
            'num_units_color_predictor': 16, 'predict_visibility': False}
    configs = {'data_loader': {'ndc': False}, 'model': {'white_bkgd': False}, 'database': 'synthetic'}
    tm = RT.CpDecomposedTensor('coarse_model', configs, tcfg, {'bounding_box': bbox})
    tm.update_tensor_params(res, torch.tensor(bbox))
    tm.vectors_density = tm.create_decomposed_tensor([5], res, 0.1)
    tm.vectors_color = tm.create_decomposed_tensor([6], res, 0.1)
    with torch.no_grad():
        for prm in tm.vectors_density:
            prm.copy_(torch.randn(prm.shape, generator=g) * 0.4 + 0.5)
        for prm in tm.vectors_color:
            prm.copy_(torch.randn(prm.shape, generator=g) * 0.5)
        for prm in list(tm.basis_matrix_color.parameters()) + list(tm.color_predictor.parameters()):
            prm.copy_(torch.randn(prm.shape, generator=g) * 0.3)
    tm.train()
    n = 10
    o = torch.zeros(n, 3)
    o[:, 2] = -3.0
    o[:, :2] = torch.rand(n, 2, generator=g) * 0.6 - 0.3
    d = torch.randn(n, 3, generator=g) * 0.15
    d[:, 2] = 1.0
    d = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    u = torch.rand(n, 1, generator=g)
    fake = types.SimpleNamespace(ndc=False, training=True,
                                 configs={'model': {'perturb': True, 'lindisp': False}},
                                 model_configs={'near': 0.5, 'far': 6.0})
    with patched_rand([u]):
        z = RT.SimpleTensoRF.get_z_vals_coarse(fake, {'pixel_id': torch.zeros(n, 3)},
                                               {'rays_o': o, 'rays_d': d}, tm)
    pts = o[:, None, :] + d[:, None, :] * z[:, :, None]
    vdir = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    inp = {'pts': pts, 'z_vals': z, 'rays_o': o, 'rays_d': d, 'view_dirs': vdir}
    with patched_rand([torch.tensor([0.25])]):       # white-background coin: rand < 0.5 -> white
        ret = tm(inp, retraw=True)
    tg = torch.Generator().manual_seed(33)
    loss = 0
    out = {}
    for k in ('rgb', 'depth', 'acc'):
        c = torch.randn(ret[k].shape, generator=tg)
        out[f'cot_{k}'] = c.numpy()
        loss = loss + torch.sum(ret[k] * c)
    loss.backward()
    out.update({'res': res.numpy(), 'bbox': np.array(bbox, np.float32), 'u': u.numpy(), 'rays_o': o.numpy(),
                'rays_d': d.numpy(), 'z': z.numpy(), 'step_size': tm.step_size.numpy(),
                'num_samples': tm.num_samples.numpy()})
    for i in range(3):
        out[f'lines_density.{i}'] = tm.vectors_density[i].detach().numpy()[0]
        out[f'lines_color.{i}'] = tm.vectors_color[i].detach().numpy()[0]
        out[f'grad_lines_density.{i}'] = tm.vectors_density[i].grad.numpy()[0]
        out[f'grad_lines_color.{i}'] = tm.vectors_color[i].grad.numpy()[0]
    out['basis_matrix_color.weight'] = tm.basis_matrix_color.weight.detach().numpy()
    out['grad_basis_matrix_color.weight'] = tm.basis_matrix_color.weight.grad.numpy()
    for k, prm in tm.color_predictor.named_parameters():
        out['color_predictor.' + k] = prm.detach().numpy()
        out['grad_color_predictor.' + k] = prm.grad.numpy()
    for k, v in ret.items():
        out['out_' + k] = v.detach().numpy()
    return out


def losses_case():
    """The reference's per-ray losses on random inputs with autograd gradients:
    MassConcentrationLoss06.compute_entropy_loss (64 and 67 samples, 5 bins),
    SparseDepthMSE14.compute_depth_loss, CoarseFineConsistencyLoss33.compute_loss and
    AugmentationsDepthLoss11.compute_depth_mse."""
    from loss_functions import AugmentationsDepthLoss11 as LAD
    from loss_functions import CoarseFineConsistencyLoss33 as LCF
    from loss_functions import MassConcentrationLoss06 as LMC
    from loss_functions import SparseDepthMSE14 as LSD
    g = torch.Generator().manual_seed(31)
    out = {}
    n = 40
    mask = torch.rand(n, generator=g) < 0.7
    out['mask'] = mask.numpy()
    for s in (64, 67):
        w = (torch.rand(n, s, generator=g) * 0.05).requires_grad_(True)
        mc = LMC.MassConcentrationLoss({'model': {}}, {'num_bins': 5})
        loss = mc.compute_entropy_loss(w, mask, False)['loss_value']
        loss.backward()
        out[f'mc{s}_weights'] = w.detach().numpy()
        out[f'mc{s}_loss'] = loss.detach().numpy()
        out[f'mc{s}_grad'] = w.grad.numpy()
    pred = (torch.rand(n, generator=g) * 4 + 2).requires_grad_(True)
    true = torch.rand(n, generator=g) * 4 + 2
    loss = LSD.SparseDepthMSE.compute_depth_loss(pred, true, mask, False)['loss_value']
    loss.backward()
    out.update(sd_pred=pred.detach().numpy(), sd_true=true.numpy(), sd_loss=loss.detach().numpy(),
               sd_grad=pred.grad.numpy())
    dc = (torch.rand(n, generator=g) * 4 + 2).requires_grad_(True)
    df = (torch.rand(n, generator=g) * 4 + 2).requires_grad_(True)
    cf = LCF.CoarseFineConsistencyLoss({'model': {'coarse_model': {}, 'fine_model': {}}, 'data_loader': {'ndc': False}},
                                       {})
    loss = cf.compute_loss({'target_rgb': torch.zeros(n, 3)}, {'depth_coarse': dc, 'depth_fine': df}, None,
                           False)['loss_value']
    loss.backward()
    out.update(cf_coarse=dc.detach().numpy(), cf_fine=df.detach().numpy(), cf_loss=loss.detach().numpy(),
               cf_grad_coarse=dc.grad.numpy(), cf_grad_fine=df.grad.numpy())
    d1 = (torch.rand(n, generator=g) * 4 + 2).requires_grad_(True)
    d2 = torch.rand(n, generator=g) * 4 + 2
    loss, _ = LAD.AugmentationsDepthLoss.compute_depth_mse(d1.clone(), d2.clone(), mask)
    loss.backward()
    out.update(ad_pred=d1.detach().numpy(), ad_target=d2.numpy(), ad_loss=loss.detach().numpy(),
               ad_grad=d1.grad.numpy())
    return out


def reprojection_case():
    """AugmentationsDepthLoss11.compute_loss_nerf on 4 forward-facing 40x30 views
    (random images, distinct camera origins) and 300 rays through random pixels,
    with depths near the scene plane: masks (from the loss maps), loss, gradients."""
    from loss_functions import AugmentationsDepthLoss11 as LAD
    g = torch.Generator().manual_seed(41)
    v, h, w = 4, 30, 40
    images = torch.rand(v, h, w, 3, generator=g)
    # a smooth scene so nearby views see similar patches for the right depth
    yy, xx = torch.meshgrid(torch.arange(h).float(), torch.arange(w).float(), indexing='ij')
    base = torch.stack([torch.sin(xx / 5), torch.cos(yy / 4), torch.sin((xx + yy) / 7)], -1) * 0.5 + 0.5
    images = 0.9 * base[None].expand(v, h, w, 3) + 0.1 * images
    poses = torch.eye(4).repeat(v, 1, 1)
    poses[:, :3, 3] = torch.tensor([[0.0, 0.0, 0.0], [0.06, 0.0, 0.0], [0.0, 0.05, 0.01], [-0.07, 0.02, 0.0]])
    k = torch.tensor([[30.0, 0.0, w / 2.0], [0.0, 30.0, h / 2.0], [0.0, 0.0, 1.0]])
    intr = k[None].repeat(v, 1, 1)
    n = 300
    img = torch.randint(0, v, (n,), generator=g)
    px = torch.randint(0, w, (n,), generator=g)
    py = torch.randint(0, h, (n,), generator=g)
    pid = torch.stack([img, px, py], -1)
    rays_o, rays_d = CU.get_rays_tr(pid, intr[img], poses[img], False)
    d1 = (1.5 + torch.rand(n, generator=g) * 2).requires_grad_(True)
    d2 = (1.5 + torch.rand(n, generator=g) * 2).requires_grad_(True)
    loss_fn = LAD.AugmentationsDepthLoss({'model': {}}, {'patch_size': [5, 5], 'rmse_threshold': 0.2})
    mask = torch.ones(n, dtype=torch.bool)
    # record the masks compute_loss_nerf hands to compute_depth_mse (mask2 first, then mask1)
    seen = []
    orig = LAD.AugmentationsDepthLoss.compute_depth_mse

    def spy(pred_depth, gt_depth, mask=None):
        seen.append(mask.clone())
        return orig(pred_depth, gt_depth, mask)

    LAD.AugmentationsDepthLoss.compute_depth_mse = staticmethod(spy)
    try:
        loss, map1, map2 = loss_fn.compute_loss_nerf(d1.clone(), d2.clone(), mask, rays_o, rays_d, poses, images,
                                                     pid, intr, (h, w))
    finally:
        LAD.AugmentationsDepthLoss.compute_depth_mse = orig
    loss.backward()
    return dict(images=images.numpy(), poses=poses.numpy(), k=k.numpy(), pixel_ids=pid.numpy().astype(np.int32),
                rays_o=rays_o.numpy(), rays_d=rays_d.numpy(), depth1=d1.detach().numpy(), depth2=d2.detach().numpy(),
                loss=loss.detach().numpy(), mask1=seen[1].numpy(), mask2=seen[0].numpy(),
                grad1=d1.grad.numpy(), grad2=d2.grad.numpy())


def coarse_fine_case():
    """CoarseFineConsistencyLoss34.compute_loss on the reprojection case's 4 views
    and 300 rays with coarse / fine depths (some rays reproject outside the image
    with both depths, where AugmentationsDepthLoss11 would add its both-invalid
    rule), 40 of them sparse-depth rays: masks (from the spy on compute_depth_mse),
    loss and autograd gradients into both depths."""
    from loss_functions import CoarseFineConsistencyLoss34 as LCF
    g = torch.Generator().manual_seed(43)
    v, h, w = 4, 30, 40
    images = torch.rand(v, h, w, 3, generator=g)
    yy, xx = torch.meshgrid(torch.arange(h).float(), torch.arange(w).float(), indexing='ij')
    base = torch.stack([torch.sin(xx / 5), torch.cos(yy / 4), torch.sin((xx + yy) / 7)], -1) * 0.5 + 0.5
    images = 0.9 * base[None].expand(v, h, w, 3) + 0.1 * images
    poses = torch.eye(4).repeat(v, 1, 1)
    poses[:, :3, 3] = torch.tensor([[0.0, 0.0, 0.0], [0.06, 0.0, 0.0], [0.0, 0.05, 0.01], [-0.07, 0.02, 0.0]])
    k = torch.tensor([[30.0, 0.0, w / 2.0], [0.0, 30.0, h / 2.0], [0.0, 0.0, 1.0]])
    intr = k[None].repeat(v, 1, 1)
    n = 300
    img = torch.randint(0, v, (n,), generator=g)
    px = torch.randint(0, w, (n,), generator=g)
    py = torch.randint(0, h, (n,), generator=g)
    pid = torch.stack([img, px, py], -1)
    rays_o, rays_d = CU.get_rays_tr(pid, intr[img], poses[img], False)
    dc = 1.5 + torch.rand(n, generator=g) * 2
    df = 1.5 + torch.rand(n, generator=g) * 2
    dc[:20] = 0.05          # very near: both reprojections far outside the image
    df[:20] = 0.04
    dc, df = dc.requires_grad_(True), df.requires_grad_(True)
    sd = torch.zeros(n, dtype=torch.bool)
    sd[-40:] = True
    nerf = ~sd
    configs = {'model': {'coarse_model': {}, 'fine_model': {}}, 'data_loader': {'sparse_depth': {}}}
    loss_fn = LCF.CoarseFineConsistencyLoss(configs, {'patch_size': [5, 5], 'rmse_threshold': 0.2})
    seen = []
    orig = LCF.CoarseFineConsistencyLoss.compute_depth_mse.__func__

    def spy(cls, pred_depth, gt_depth, mask=None):
        seen.append(None if mask is None else mask.clone())
        return orig(cls, pred_depth, gt_depth, mask)

    LCF.CoarseFineConsistencyLoss.compute_depth_mse = classmethod(spy)
    try:
        out = loss_fn.compute_loss(
            {'target_rgb': torch.zeros(n, 3), 'common_data': {'images': images, 'resolution': (h, w)},
             'indices_mask_nerf': nerf, 'indices_mask_sparse_depth': sd, 'pixel_id': pid},
            {'rays_o': rays_o, 'rays_d': rays_d, 'depth_coarse': dc, 'depth_fine': df, 'intrinsics': intr,
             'extrinsics_all': poses}, None)
    finally:
        LCF.CoarseFineConsistencyLoss.compute_depth_mse = classmethod(orig)
    out['loss_value'].backward()
    return dict(images=images.numpy(), poses=poses.numpy(), k=k.numpy(), pixel_ids=pid.numpy().astype(np.int32),
                rays_o=rays_o.numpy(), rays_d=rays_d.numpy(), depth_coarse=dc.detach().numpy(),
                depth_fine=df.detach().numpy(), nerf_mask=nerf.numpy(), sd_mask=sd.numpy(),
                loss=out['loss_value'].detach().numpy(), mask1=seen[1].numpy(), mask2=seen[0].numpy(),
                grad_coarse=dc.grad.numpy(), grad_fine=df.grad.numpy())


def tv_case():
    """TotalVariationLoss04 on random grids with autograd gradients:
    compute_tv_loss on three VM-like planes of unequal shapes (one with a single
    row), on three CP-like lines (1, R, L, 1), and the iteration weight of a
    configured instance."""
    from loss_functions import TotalVariationLoss04 as LTV
    g = torch.Generator().manual_seed(47)
    out = {}
    sets = {'vm': [(1, 6, 17, 23), (1, 4, 9, 31), (1, 5, 1, 12)],
            'cp': [(1, 7, 29, 1), (1, 3, 40, 1), (1, 5, 11, 1)]}
    iter_weight = 0.37
    for tag, shapes in sets.items():
        comps = [(torch.randn(*sh, generator=g) * 0.1).requires_grad_(True) for sh in shapes]
        loss = LTV.TotalVariationLoss.compute_tv_loss(comps, iter_weight, False)['loss_value']
        loss.backward()
        for i, c in enumerate(comps):
            out[f'{tag}_comp{i}'] = c.detach().numpy()
            out[f'{tag}_grad{i}'] = c.grad.numpy()
        out[f'{tag}_loss'] = loss.detach().numpy()
    out['iter_weight'] = np.array(iter_weight)
    cfg = {'model': {}, 'num_iterations': 30000,
           'optimizers': [{'name': 'optimizer_main', 'lr_decay_ratio': 0.1, 'lr_decay_iters': None}]}
    tv = LTV.TotalVariationLoss(cfg, {'weight_density': 1.0, 'weight_color': 1.0})
    out['decay_iter_num'] = np.array(1234)
    out['decay_weight'] = np.array(tv.get_iter_weight(1234))
    return out


def camera_learners_case():
    """Learnt camera poses (ExtrinsicsLearner, SimpleNeRF17.py:817-912) and
    intrinsics (IntrinsicsLearner, SimpleNeRF17.py:788-814): seeded axis-angle
    and translation deltas on 5 frames, the composed extrinsics for 7 frame ids
    (repeats included), and the gradients of a fixed weighted sum of them with
    respect to the deltas."""
    g = np.random.default_rng(21)
    n = 5
    init = np.tile(np.eye(4), (n, 1, 1))
    init[:, :3, :3] = np.linalg.qr(g.standard_normal((n, 3, 3)))[0]
    init[:, :3, 3] = g.standard_normal((n, 3))
    intr = np.tile(np.array([[400.0, 0, 252.0], [0, 400.0, 189.0], [0, 0, 1.0]]), (n, 1, 1))
    r = (g.standard_normal((n, 3)) * 0.3).astype(np.float32)
    r[2] = 0.0   # the zero rotation (the 1e-15 guard of the angle)
    t = (g.standard_normal((n, 3)) * 0.2).astype(np.float32)
    ids = np.array([0, 2, 4, 1, 2, 3, 0])
    wsum = g.standard_normal((len(ids), 4, 4)).astype(np.float32)
    el = RN.ExtrinsicsLearner(init, learn_rotation=True, learn_translation=True)
    with torch.no_grad():
        el.r.copy_(torch.from_numpy(r))
        el.t.copy_(torch.from_numpy(t))
    ext = el(torch.from_numpy(ids))
    (ext * torch.from_numpy(wsum)).sum().backward()
    il = RN.IntrinsicsLearner(intr, learn_focal=False)
    return {'init_extrinsics': init, 'init_intrinsics': intr, 'r': r, 't': t, 'ids': ids, 'wsum': wsum,
            'extrinsics': ext.detach().numpy(), 'grad_r': el.r.grad.numpy(), 'grad_t': el.t.grad.numpy(),
            'intrinsics': il(torch.from_numpy(ids)).numpy()}


def main():
    cases = {
        'nerf_sampling': sampling_case,
        'nerf_pe': pe_case,
        'nerf_mlp': mlp_case,
        'nerf_composite': composite_case,
        'rays': rays_case,
        'nerf_render': lambda: render_case(16, 64, 128, 3, mlp_cfg(ns=64), mlp_cfg(ns=128)),
        'nerf_train_grads': lambda: render_case(16, 16, 32, 5, mlp_cfg(width=32, wv=16, ns=16),
                                                mlp_cfg(width=32, wv=16, ns=32), white=True, with_grads=True),
        'nerf_ndc_pair': lambda: render_case(
            12, 64, 128, 9, mlp_cfg(ns=64), mlp_cfg(ns=128), ndc=True,
            augs=[{'name': 'views_augmentation', 'coarse_model': mlp_cfg(lp=4, views=False, vdr=False)}],
            aug_seeds=[77]),
        'tensorf': tensorf_case,
        'tensorf_ndc': tensorf_ndc_case,
        'tensorf_realistic': tensorf_realistic_case,
        'tensorf_e2e': tensorf_e2e_case,
        'tensorf_cp': tensorf_cp_case,
        'state_dicts': state_dict_case,
        'output_keys': output_keys_case,
        'tensorf_maintenance': tensorf_maintenance_case,
        'losses': losses_case,
        'reprojection': reprojection_case,
        'coarse_fine': coarse_fine_case,
        'tv': tv_case,
        'camera_learners': camera_learners_case,
    }
    only = sys.argv[1:]
    for name, fn in cases.items():
        if only and name not in only:
            continue
        data = fn()
        data['torch_version'] = np.array(torch.__version__)
        path = os.path.join(HERE, f'{name}.npz')
        np.savez_compressed(path, **data)
        print(f'{name}: {len(data)} arrays, {os.path.getsize(path) / 1024:.1f} KiB')


if __name__ == '__main__':
    main()
