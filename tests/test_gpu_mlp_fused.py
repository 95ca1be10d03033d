"""The fused forward of the 16-bit NeRF MLP (one tcgen05 kernel from the
encodings to the heads, srf_nerf_mlp_fused_path) against the per-layer kernels
and the float64 oracle.

Both paths form the same products in the same order and round the same
activations; the head dot products (sigma, rgb) sum their 32-column partials in
another order, so sigma / rgb agree within 1e-6 relative; the share of
bitwise-equal outputs is printed.  The training forward (mode 2) also stores
every activation and ReLU mask the backward reads: gradients after it match the
per-layer path within 1e-4 relative L2 -- the last-bit differences of the heads
reach the 16-bit rounding of the backward's dZ, and the atomically summed bias
gradients differ in summation order (the bar vs the float64 oracle is 1e-2).
Layouts the kernel does not cover (the points-augmentation variant) run per
layer in every mode.  Sizes cover one row, partial and exact tiles, and more
tiles than a persistent CTA takes in one round."""
import numpy as np
import pytest
import torch

from oracle import nerf as on

pytestmark = pytest.mark.gpu
DEV = 'cuda'

SPECS = {
    'main': dict(),
    'aug_l4_noview': dict(points_pe_degree=4, use_view_dirs=False, view_dependent_rgb=False),
    'depth4_no_skip': dict(points_net_depth=4, skip_layer=-1),
    'points_aug': dict(points_sigma_pe_degree=3),
}


@pytest.fixture(scope='module', autouse=True)
def built():
    from simple_rf_gb300 import build as b
    b.build()


def _mode(mode):
    from simple_rf_gb300 import _lib
    return _lib.load().srf_nerf_mlp_fused_path(mode)


def _ospec(kw):
    return on.MlpSpec(points_pe_degree=kw.get('points_pe_degree', 10), use_view_dirs=kw.get('use_view_dirs', True),
                      view_dependent_rgb=kw.get('view_dependent_rgb', True),
                      points_sigma_pe_degree=kw.get('points_sigma_pe_degree'),
                      points_net_depth=kw.get('points_net_depth', 8))


def _inputs(m, div, seed):
    rng = np.random.default_rng(seed)
    pts = (rng.standard_normal((m, 3)) * 0.7).astype(np.float32)
    vd = rng.standard_normal(((m + div - 1) // div, 3))
    vd = (vd / np.linalg.norm(vd, axis=1, keepdims=True)).astype(np.float32)
    noise = (rng.standard_normal(m) * 0.3).astype(np.float32)
    return pts, vd, noise


def _run(spec, precision, params, pts, vd, div, noise, mode, grad, cot=None):
    from simple_rf_gb300 import _lib
    from simple_rf_gb300 import functional as F
    prev = _mode(mode)
    try:
        ps = [p.detach().clone().requires_grad_(grad) for p in params]
        tp = torch.from_numpy(pts).to(DEV)
        tv = torch.from_numpy(vd).to(DEV) if spec.use_view_dirs else None
        tn = torch.from_numpy(noise).to(DEV) if noise is not None else None
        with torch.set_grad_enabled(grad):
            sigma, rgb = F.NerfMlpFunction.apply(spec, _lib.PRECISIONS[precision], tp, tv, div, tn, *ps)
            if grad:
                cs, cr = cot
                ((sigma * torch.from_numpy(cs).to(DEV)).sum() + (rgb * torch.from_numpy(cr).to(DEV)).sum()).backward()
        torch.cuda.synchronize()
        out = (sigma.detach().cpu().numpy(), rgb.detach().cpu().numpy())
        grads = [p.grad.double().cpu().numpy() for p in ps] if grad else None
        return out, grads
    finally:
        _mode(prev)


def _params(spec, kw, seed):
    """Xavier weights and small random biases (the bias adds are exercised)."""
    p64 = on.xavier_params(_ospec(kw), seed, np.float64)
    rng = np.random.default_rng(seed + 1)
    for k in p64:
        if k.endswith('bias'):
            p64[k] = (rng.standard_normal(p64[k].shape) * 0.1).astype(np.float32).astype(np.float64)
    return p64, [torch.from_numpy(p64[k].astype(np.float32)).to(DEV) for k in spec.param_names]


@pytest.mark.parametrize('precision', ['bf16', 'fp16'])
@pytest.mark.parametrize('name', list(SPECS))
@pytest.mark.parametrize('m', [1, 129, 5000, 200003])
def test_fused_forward_matches_per_layer(name, precision, m):
    from simple_rf_gb300 import functional as F
    kw = SPECS[name]
    spec = F.MlpSpec(**kw)
    _, params = _params(spec, kw, 5)
    div = 64
    pts, vd, noise = _inputs(m, div, m)
    (s0, r0), _ = _run(spec, precision, params, pts, vd, div, noise, 0, False)
    (s1, r1), _ = _run(spec, precision, params, pts, vd, div, noise, 1, False)
    same = np.mean(np.concatenate([(s0 == s1), (r0 == r1).ravel()]))
    print(name, precision, m, 'share of outputs bitwise equal to the per-layer path', same)
    np.testing.assert_allclose(r1, r0, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(s1, s0, rtol=1e-6, atol=1e-6 * max(1.0, float(np.abs(s0).max())))
    assert np.isfinite(s1).all() and np.isfinite(r1).all()


@pytest.mark.parametrize('precision', ['bf16', 'fp16'])
@pytest.mark.parametrize('name', list(SPECS))
def test_fused_training_forward_gives_the_per_layer_gradients(name, precision):
    from simple_rf_gb300 import functional as F
    kw = SPECS[name]
    spec = F.MlpSpec(**kw)
    _, params = _params(spec, kw, 9)
    div, m = 64, 64 * 97 + 13
    pts, vd, noise = _inputs(m, div, 3)
    rng = np.random.default_rng(4)
    cot = (rng.standard_normal(m).astype(np.float32), rng.standard_normal((m, 3)).astype(np.float32))
    (s0, r0), g0 = _run(spec, precision, params, pts, vd, div, noise, 0, True, cot)
    (s2, r2), g2 = _run(spec, precision, params, pts, vd, div, noise, 2, True, cot)
    np.testing.assert_allclose(r2, r0, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(s2, s0, rtol=1e-6, atol=1e-6 * max(1.0, float(np.abs(s0).max())))
    a = np.concatenate([g.ravel() for g in g0])
    b = np.concatenate([g.ravel() for g in g2])
    rel = np.linalg.norm(a - b) / np.linalg.norm(a)
    print(name, precision, 'gradients, fused training forward vs per layer: rel-L2', rel,
          'bitwise-equal share', float(np.mean(a == b)))
    assert rel < 1e-4, rel


@pytest.mark.parametrize('precision', ['bf16', 'fp16'])
def test_fused_forward_against_fp64_oracle(precision):
    """Forward-only fused path, benchmark network (8 x 256, skip, view branch),
    8192 samples of 128 rays: rgb within 2e-3 max-abs of the float64 oracle."""
    from simple_rf_gb300 import functional as F
    spec = F.MlpSpec()
    p64, params = _params(spec, {}, 20)
    div, m = 64, 8192
    pts, vd, _ = _inputs(m, div, 21)
    (s1, r1), _ = _run(spec, precision, params, pts, vd, div, None, 1, False)
    rs, rr, _ = on.mlp_forward(p64, _ospec({}), pts.astype(np.float64), np.repeat(vd.astype(np.float64), div, 0))
    err = float(np.abs(r1 - rr).max())
    print(precision, 'fused forward rgb max-abs vs float64', err)
    assert err < 2e-3
    assert np.abs(s1 - rs[:, 0]).max() < 2e-2 * max(1.0, np.abs(rs).max())


def test_fused_path_switch_round_trips():
    prev = _mode(-1)
    assert prev in (0, 1, 2)
    assert _mode(0) == prev
    assert _mode(-1) == 0
    _mode(prev)
    assert _mode(-1) == prev


@pytest.mark.parametrize('mode', [0, 1])
@pytest.mark.parametrize('blowup', [1.0, 30.0])
def test_fp16_overflow_sets_found_inf(mode, blowup):
    """FP16 forward-only calls report activations beyond the format's range in the
    loss scaler's found_inf, the fused kernel (mode 1) as the per-layer kernels
    (mode 0): weights scaled by 30 push the trunk past 65504 within a few layers;
    the unscaled net leaves the flag clear."""
    import ctypes
    from simple_rf_gb300 import _lib
    from simple_rf_gb300 import functional as F
    spec = F.MlpSpec()
    _, params = _params(spec, {}, 12)
    params = [p * blowup if name.endswith('weight') else p for name, p in zip(spec.param_names, params)]
    div, m = 64, 64 * 40 + 7
    pts, vd, _ = _inputs(m, div, 13)
    tp, tv = torch.from_numpy(pts).to(DEV), torch.from_numpy(vd).to(DEV)
    sigma = torch.empty(m, device=DEV)
    rgb = torch.empty(m, 3, device=DEV)
    prec = _lib.PRECISIONS['fp16']
    wsb = spec.workspace_bytes(m, prec, False)
    ws = torch.empty(wsb, dtype=torch.uint8, device=DEV)
    scaler = torch.zeros(4, dtype=torch.int32, device=DEV)
    scaler[:2] = torch.tensor([65536.0, 1 / 65536.0], device=DEV).view(torch.int32)
    arr = (ctypes.c_void_p * len(params))(*[t.data_ptr() for t in params])
    prev = _mode(mode)
    try:
        _lib.call('srf_nerf_mlp_forward', ctypes.byref(spec.desc), arr, ctypes.c_void_p(tp.data_ptr()),
                  ctypes.c_void_p(tv.data_ptr()), div, m, None, ctypes.c_void_p(sigma.data_ptr()),
                  ctypes.c_void_p(rgb.data_ptr()), prec, 0, ctypes.c_void_p(ws.data_ptr()), wsb,
                  ctypes.c_void_p(scaler.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
    finally:
        _mode(prev)
    assert int(scaler[2].item()) == (1 if blowup > 1 else 0), (mode, blowup, int(scaler[2].item()))
