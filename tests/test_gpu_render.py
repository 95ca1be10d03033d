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
