"""The oracle's hand-derived backward against float64 central finite differences.

The GPU kernels' gradients are checked against the oracle's backward; this pins
that backward itself to finite differences of the float64 forward, on a 64-ray
subset of the training-step workload (64 stratified + 128 inverse-CDF samples,
8x256 coarse and fine nets, white background, rgb MSE + 0.1 L1 depth on 25% of
the rays).  Depths are held fixed as the reference's detach does
(SimpleNeRF17.py:368).  The sigma-head bias is 0.5 so no ray sits on the
non-NDC last-sample step (delta = 1e10 |d|, SimpleNeRF17.py:489-492).

Bar: |<g, v> - FD| <= 2e-6 |FD| along gradient directions and <= 2e-6 ||g||
along a random unit direction.  The step is eps = 1e-6 along unit directions:
larger steps cross ReLU kinks of the 2M hidden pre-activations (at eps = 1e-4
the difference quotient is off by up to 7e-5), and at 1e-6 float64 rounding of
the loss contributes ~1e-10; the measured agreement is 1e-8 ... 3e-7.
"""
import numpy as np

from oracle import fd
from oracle import nerf as on

N_RAYS, SC, SF = 64, 64, 128
KEYS = ('pts_linears.0.weight', 'pts_linears.5.weight', 'pts_output_linear.weight', 'pts_output_linear.bias',
        'feature_linear.weight', 'views_linears.0.weight', 'views_output_linear.bias')


def _problem():
    rng = np.random.default_rng(5)
    spec = on.MlpSpec()
    p = {tag: on.xavier_params(spec, s, np.float64) for tag, s in (('coarse', 11), ('fine', 12))}
    for prm in p.values():
        prm['pts_output_linear.bias'][:] = 0.5
    o = rng.standard_normal((N_RAYS, 3)) * 0.1
    d = rng.standard_normal((N_RAYS, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    t_rgb = rng.random((N_RAYS, 3))
    t_d = rng.random(N_RAYS) * 4 + 2
    mask = np.zeros(N_RAYS)
    mask[:N_RAYS // 4] = 1
    u_c, u_f = rng.random((N_RAYS, SC)), rng.random((N_RAYS, SF))
    return spec, p, (o, d, t_rgb, t_d, mask, u_c, u_f)


def test_oracle_backward_matches_fp64_central_differences():
    spec, p, (o, d, t_rgb, t_d, mask, u_c, u_f) = _problem()
    ret, caches = on.render_rays(p['coarse'], p['fine'], spec, spec, o, d, 2.0, 6.0, SC, SF, u_c, u_f,
                                 white_bkgd=True, pts_fp32=True)
    _, g = on.train_loss(ret, t_rgb, t_d, mask)
    grads = on.backward_render(p, {'coarse': spec, 'fine': spec}, caches, g, N_RAYS)
    rng = np.random.default_rng(0)
    for tag in ('coarse', 'fine'):
        z = ret[f'z_vals_{tag}']

        def loss(prm):
            return fd.level_loss(prm, spec, o, d, z, t_rgb, t_d, mask)
        gnorm = np.sqrt(sum(float(np.sum(v * v)) for v in grads[tag].values()))
        for name, v in fd.unit_directions(grads[tag], KEYS, rng):
            num = fd.directional_derivative(loss, p[tag], v, 1e-6)
            ana = fd.dot(grads[tag], v)
            scale = gnorm if name == 'random' else abs(num)
            assert abs(ana - num) <= 2e-6 * scale, (tag, name, ana, num)
