"""Edge cases of the hot path against the oracle: ray lengths on either side of
every compositing kernel variant (1 ... 5000 samples: register-resident rounds
up to 256 samples, shared-memory scans beyond), empty batches, all-zero coarse
weights (the pdf floor and the denom < 1e-5 rule of SimpleNeRF17.py:400-413),
and TensoRF rays that miss the bounding box (no valid samples).

Tolerances as in tests/test_gpu_kernels.py: 1e-5 relative (absolute floor 1e-6
of the value range) on compositing outputs, 1e-5 relative L2 on its adjoints
(5e-5 for rays of more than 2048 samples, see below); fine samples 1e-5.
"""
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


def t(x):
    return torch.from_numpy(np.ascontiguousarray(x, np.float32)).to(DEV)


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize('s', [1, 2, 31, 33, 64, 100, 192, 255, 256, 257, 1039, 5000])
@pytest.mark.parametrize('ndc', [False, True])
def test_composite_every_ray_length(s, ndc):
    from simple_rf_gb300 import functional as F
    rng = np.random.default_rng(s)
    nr = 19
    sigma = np.maximum(rng.standard_normal((nr, s)) * 3, 0).astype(np.float32)
    sigma[0] = 0                      # a fully transparent ray
    sigma[1, s // 2:] = 1e4           # an opaque wall half way
    rgb = rng.random((nr, s, 3), dtype=np.float32)
    kw = {}
    if ndc:
        o = np.zeros((nr, 3), np.float32)
        o[:, :2] = rng.uniform(-1, 1, (nr, 2))
        o[:, 2] = -1
        d = np.stack([rng.uniform(-.2, .2, nr), rng.uniform(-.2, .2, nr), -rng.uniform(.8, 1.2, nr)],
                     1).astype(np.float32)
        f = np.full(nr, 400.0, np.float32)
        _, dn = on.ndc_rays(o, d, 378, 504, f, f, 1.0)
        z = np.sort(rng.random((nr, s), dtype=np.float32), 1)
        z[2, -1] = 1.0                # the last NDC sample exactly at infinity
        kw = dict(ndc=True, rays_o=o, rays_d_ndc=dn.astype(np.float32))
    else:
        d = rng.standard_normal((nr, 3)).astype(np.float32)
        z = (2 + 4 * np.sort(rng.random((nr, s), dtype=np.float32), 1)).astype(np.float32)
    ref, cache = on.composite_forward(sigma, rgb, z, d, white_bkgd=True, **kw)
    sg, rg = t(sigma).requires_grad_(True), t(rgb).requires_grad_(True)
    got = F.composite(sg, rg, t(z), t(d), white_bkgd=True, ndc=ndc,
                      rays_o=t(kw['rays_o']) if ndc else None, rays_d_ndc=t(kw['rays_d_ndc']) if ndc else None)
    # Rays longer than any configuration (5000 samples): the float32 running
    # product of 5000 transmittance factors drifts up to ~3e-5 from the oracle's
    # double-accumulated cumprod (torch's own CUDA cumprod accumulates in float
    # too); every length up to 2048 holds 1e-5.
    # NDC metric depth: the far samples (z_ndc -> 1, metric depth up to ~1e4)
    # carry alphas 1 - exp(-x) with x ~ 1e-4, which float32 holds to ~5e-4
    # relative, yet a weight of 1e-5 there is ~10% of a ray's depth: float32
    # evaluations of the reference formula (numpy on two hosts, the GPU) spread
    # by ~1.5e-5 around the float64 value (the depth_var terms are worse).
    long_ray = s > 2048
    for k, v in ref.items():
        if k.startswith('depth_var'):
            rtol = 2e-4
        elif long_ray or (ndc and k == 'depth'):
            rtol = 5e-5
        else:
            rtol = 1e-5
        np.testing.assert_allclose(got[k].detach().cpu().numpy(), v, rtol=rtol,
                                   atol=1e-6 * max(1.0, float(np.abs(v).max())), err_msg=f'{k} s={s}')
    cot = {k: rng.standard_normal(ref[k].shape).astype(np.float32) for k in ref if k not in ('alpha', 'visibility')}
    sum((got[k] * t(c)).sum() for k, c in cot.items()).backward()
    ds, dr = on.composite_backward(cache, cot)
    # float32 transmittance products over 1000+ samples drift ~2e-6 from the
    # oracle's double-accumulated cumprod: 1e-5 holds for every length
    bar = 5e-5 if long_ray else 1e-5
    assert rel_l2(sg.grad.cpu().numpy(), ds) < bar, s
    assert rel_l2(rg.grad.cpu().numpy(), dr) < bar, s


def test_composite_without_colour_and_with_per_ray_background():
    """rgb NULL (the TensoRF density pass) and a per-ray white-background coin."""
    from simple_rf_gb300 import functional as F
    rng = np.random.default_rng(3)
    nr, s = 40, 192
    sigma = np.maximum(rng.standard_normal((nr, s)), 0).astype(np.float32)
    d = rng.standard_normal((nr, 3)).astype(np.float32)
    z = (2 + 4 * np.sort(rng.random((nr, s), dtype=np.float32), 1)).astype(np.float32)
    coin = rng.random(nr) < 0.5
    got = F.composite(t(sigma), None, t(z), t(d), distance_scale=25.0,
                      white_per_ray=torch.from_numpy(coin).to(DEV))
    ref, _ = on.composite_forward(sigma, np.zeros((nr, s, 3), np.float32), z, d, distance_scale=25.0)
    exp_rgb = ref['rgb'] + np.where(coin[:, None], 1 - ref['acc'][:, None], 0)
    np.testing.assert_allclose(got['rgb'].cpu().numpy(), exp_rgb, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(got['weights'].cpu().numpy(), ref['weights'], rtol=1e-5, atol=1e-6)


def test_empty_batches():
    """Zero rays / zero samples through compositing, sampling and the MLP."""
    from simple_rf_gb300 import _lib
    from simple_rf_gb300 import functional as F
    e = torch.zeros(0, 64, device=DEV)
    out = F.composite(e, torch.zeros(0, 64, 3, device=DEV), e, torch.zeros(0, 3, device=DEV), white_bkgd=True)
    assert out['rgb'].shape == (0, 3) and out['weights'].shape == (0, 64)
    z = F.fine_z(e, e, 128, torch.zeros(0, 128, device=DEV))
    assert z.shape == (0, 192)
    spec = F.MlpSpec()
    params = [torch.zeros(int(nm), device=DEV).requires_grad_(True) for nm in spec.param_numel]
    sigma, rgb = F.NerfMlpFunction.apply(spec, _lib.SRF_PRECISION_FP32, torch.zeros(0, 3, device=DEV),
                                         torch.zeros(0, 3, device=DEV), 64, None, *params)
    assert sigma.shape == (0,) and rgb.shape == (0, 3)
    (sigma.sum() + rgb.sum()).backward()
    assert all(p.grad is not None and torch.count_nonzero(p.grad) == 0 for p in params)


def test_fine_sampling_with_all_zero_coarse_weights():
    """Weights that are all zero leave only the 1e-5 pdf floor: the fine samples
    follow the uniform inverse CDF of the bins, exactly as the oracle's."""
    from simple_rf_gb300 import functional as F
    rng = np.random.default_rng(11)
    nr, sc, sf = 50, 64, 128
    zc = on.stratified_z(2.0, 6.0, nr, sc, rng.random((nr, sc), dtype=np.float32))
    w = np.zeros((nr, sc), np.float32)
    w[::2, 5] = 1e-9                  # below the floor's scale on every other ray
    u = rng.random((nr, sf), dtype=np.float32)
    got = F.fine_z(t(zc), t(w), sf, t(u)).cpu().numpy()
    ref = on.fine_z(zc, w, sf, u)
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5)
    assert np.all(np.diff(got, axis=1) >= 0)


def test_tensorf_rays_that_miss_the_box():
    """Every ray misses the bounding box: no valid samples, zero weights, white
    background; the compaction sees an empty mask.  As in the reference (whose
    sigma stays a zero tensor when no sample is valid, SimpleTensoRF09.py:1220),
    no parameter reaches the outputs."""
    from simple_rf_gb300.tensorf_model import GbVmTensor
    from simple_rf_gb300.bench_tensorf import tensor_configs
    configs = {'data_loader': {'ndc': False}, 'model': {'white_bkgd': True}}
    bbox = [[-1.5] * 3, [1.5] * 3]
    tm = GbVmTensor('coarse_model', configs, tensor_configs(32 ** 3), {'bounding_box': bbox}).to(DEV)
    n, s = 64, 100
    o = torch.zeros(n, 3, device=DEV)
    o[:, 0] = 10.0
    d = torch.zeros(n, 3, device=DEV)
    d[:, 0] = 1.0                     # pointing away from the box
    z = torch.linspace(2.0, 6.0, s, device=DEV).repeat(n, 1).contiguous()
    out = tm({'z_vals': z, 'rays_o': o, 'rays_d': d, 'view_dirs': d}, retraw=True)
    assert tm.last_sample_counts['valid'] == 0 and tm.last_sample_counts['surface'] == 0
    assert torch.count_nonzero(out['weights']) == 0
    assert torch.equal(out['rgb'], torch.ones_like(out['rgb']))
    assert not out['rgb'].requires_grad


def _exp_prefix_reference(sigma, rgb, z, d, *, white, ndc=None):
    """The exp-of-prefix-sum compositing in float64 torch on the CPU (autograd
    gives the reference gradients): y = sigma delta, alpha = 1 - exp(-y),
    T_i = exp(-sum_{j<i} y_j), w = alpha T, then the reference's sums."""
    import torch as th
    dvec = ndc['d_ndc'] if ndc else d
    inf = 1.0 if ndc else 1e10
    z1 = th.cat([z, th.full_like(z[:, :1], inf)], -1)
    delta = (z1[:, 1:] - z1[:, :-1]) * th.linalg.norm(dvec, dim=-1, keepdim=True)
    y = sigma * delta
    alpha = 1 - th.exp(-y)
    csum = th.cumsum(y, -1)
    T = th.exp(-th.cat([th.zeros_like(csum[:, :1]), csum[:, :-1]], -1))
    w = alpha * T
    acc = w.sum(-1)
    rgb_map = (w[..., None] * rgb).sum(-2)
    if white:
        rgb_map = rgb_map + (1 - acc[:, None])
    if ndc:
        oz, dz = ndc['o'][:, 2:3], d[:, 2:3]
        tn = -(1 + oz) / dz
        zm = (oz + tn * dz) / dz * (1 / (1 - z + (z == 1).double() * 1e-3) - 1) + tn
    else:
        zm = z
    depth = (w * zm).sum(-1) / (acc + 1e-6)
    return {'rgb': rgb_map, 'acc': acc, 'depth': depth, 'weights': w}


@pytest.mark.parametrize('s', [1, 33, 64, 192, 256])
@pytest.mark.parametrize('ndc', [False, True])
def test_composite_exp_prefix_transmittance(s, ndc):
    """SRF_COMPOSITE_EXP_PREFIX (T = exp of an exclusive prefix sum of sigma delta,
    the 16-bit steps' form) against the same formula in float64 torch with
    autograd: outputs within 1e-5 relative, sigma and rgb gradients within 1e-5
    relative L2; and it stays within 1e-6 of the reference's cumprod form."""
    import torch as th
    from simple_rf_gb300 import _lib
    from simple_rf_gb300 import functional as F
    rng = np.random.default_rng(100 + s)
    nr = 23
    sigma = np.maximum(rng.standard_normal((nr, s)) * 2, 0).astype(np.float32)
    rgb = rng.random((nr, s, 3), dtype=np.float32)
    extra = {}
    if ndc:
        o = np.zeros((nr, 3), np.float32)
        o[:, :2] = rng.uniform(-1, 1, (nr, 2))
        o[:, 2] = -1
        d = np.stack([rng.uniform(-.2, .2, nr), rng.uniform(-.2, .2, nr), -rng.uniform(.8, 1.2, nr)],
                     1).astype(np.float32)
        f = np.full(nr, 400.0, np.float32)
        _, dn = on.ndc_rays(o, d, 378, 504, f, f, 1.0)
        dn = dn.astype(np.float32)
        z = np.sort(rng.random((nr, s), dtype=np.float32), 1)
        extra = dict(ndc=True, rays_o=t(o), rays_d_ndc=t(dn))
        ref_ndc = {'o': th.from_numpy(o).double(), 'd_ndc': th.from_numpy(dn).double()}
    else:
        d = rng.standard_normal((nr, 3)).astype(np.float32)
        z = (2 + 4 * np.sort(rng.random((nr, s), dtype=np.float32), 1)).astype(np.float32)
        ref_ndc = None
    sg, rg = t(sigma).requires_grad_(True), t(rgb).requires_grad_(True)
    flags = _lib.SRF_COMPOSITE_WHITE_BKGD | _lib.SRF_COMPOSITE_EXP_PREFIX | (_lib.SRF_COMPOSITE_NDC if ndc else 0)
    outs = F.CompositeFunction.apply(sg, rg, t(z), t(d), extra.get('rays_o'), extra.get('rays_d_ndc'), flags, 1.0,
                                     None)
    got = dict(zip(F._COMPOSITE_OUT, outs))
    ss = th.from_numpy(sigma).double().requires_grad_(True)
    rr = th.from_numpy(rgb).double().requires_grad_(True)
    ref = _exp_prefix_reference(ss, rr, th.from_numpy(z).double(), th.from_numpy(d).double(), white=True,
                                ndc=ref_ndc)
    for k in ('rgb', 'acc', 'depth', 'weights'):
        v = ref[k].detach().numpy()
        rtol = 5e-5 if (ndc and k == 'depth') else 1e-5
        np.testing.assert_allclose(got[k].detach().cpu().numpy(), v, rtol=rtol,
                                   atol=1e-6 * max(1.0, float(np.abs(v).max())), err_msg=k)
    cot = {k: rng.standard_normal(tuple(ref[k].shape)).astype(np.float32) for k in ('rgb', 'acc', 'depth', 'weights')}
    sum((got[k] * t(c)).sum() for k, c in cot.items()).backward()
    sum((ref[k] * th.from_numpy(c).double()).sum() for k, c in cot.items()).backward()
    assert rel_l2(sg.grad.cpu().numpy(), ss.grad.numpy()) < 1e-5
    assert rel_l2(rg.grad.cpu().numpy(), rr.grad.numpy()) < 1e-5
    plain = F.composite(t(sigma), t(rgb), t(z), t(d), white_bkgd=True, **extra)
    assert float((plain['rgb'] - got['rgb']).detach().abs().max()) < 1e-6


def test_composite_exp_prefix_rejects_long_rays():
    from simple_rf_gb300 import _lib
    from simple_rf_gb300 import functional as F
    s = 300
    e = torch.rand(4, s, device=DEV)
    with pytest.raises(RuntimeError, match='UNSUPPORTED'):
        F.CompositeFunction.apply(e, torch.rand(4, s, 3, device=DEV), e.sort(1)[0] + 2, torch.rand(4, 3, device=DEV),
                                  None, None, _lib.SRF_COMPOSITE_EXP_PREFIX, 1.0, None)


@pytest.mark.parametrize('s', [64, 192, 256, 100, 4])
@pytest.mark.parametrize('flags', [0, 1, 2, 4, 6])
def test_composite_staged_matches_register_kernel(s, flags):
    """Rays of a multiple of 4 samples with 16-byte aligned inputs run the staged
    kernels (each warp's next ray copied to shared memory by bulk asynchronous
    copies while it composites the current one, lane j owning contiguous samples);
    the same inputs 4 bytes off 16-byte alignment run the register kernels that
    read global memory (lane j owning samples j, j + 32, ...).  Per sample the
    arithmetic is the same; the scans and sums group their terms differently, so
    the outputs and adjoints agree to float32 rounding: 1e-5 relative plus 1e-6 of
    the output's largest magnitude (the adjoints' differences G - R cancel).
    flags: 1 NDC, 2 white background, 4 exp-prefix transmittance."""
    import ctypes
    from simple_rf_gb300 import _lib
    from simple_rf_gb300.functional import _stream
    n = 3000
    g = torch.Generator().manual_seed(s + flags)
    sig = (torch.rand(n, s, generator=g) * 3 - 0.5).clamp_min(0)
    rgb = torch.rand(n, s, 3, generator=g)
    z = torch.sort(torch.rand(n, s, generator=g) * (0.9 if flags & 1 else 4) + (0.05 if flags & 1 else 2), 1).values
    d = torch.nn.functional.normalize(torch.randn(n, 3, generator=g), dim=-1)
    d[:, 2] = -d[:, 2].abs() - 0.5
    o = torch.randn(n, 3, generator=g) * 0.1
    o[:, 2] = -1.0
    gs = {k: torch.randn(sh, generator=g) for k, sh in (('rgb', (n, 3)), ('acc', (n,)), ('depth', (n,)),
                                                          ('depth_var', (n,)), ('weights', (n, s)))}

    def run(misalign):
        def put(x):
            flat = x.reshape(-1)
            buf = torch.zeros(flat.numel() + 4, device=DEV)
            off = 1 if misalign else 0
            buf[off:off + flat.numel()] = flat.to(DEV)
            return buf, buf[off:off + flat.numel()].view(x.shape)
        keep = []
        ins = {}
        for k, x in (('sigma', sig), ('rgb', rgb), ('z', z)):
            b, v = put(x)
            keep.append(b)
            ins[k] = v
        d_dev, o_dev = d.to(DEV).contiguous(), o.to(DEV).contiguous()
        dn = (d_dev / d_dev[:, 2:3].abs()).contiguous()
        outs = {k: torch.zeros(n, device=DEV) for k in ('acc', 'depth', 'depth_var', 'depth_ndc', 'depth_var_ndc')}
        outs['rgb_map'] = torch.zeros(n, 3, device=DEV)
        for k in ('alpha', 'visibility', 'weights', 'd_sigma'):
            outs[k] = torch.zeros(n, s, device=DEV)
        outs['d_rgb'] = torch.zeros(n, s, 3, device=DEV)
        gd = {k: v.to(DEV).contiguous() for k, v in gs.items()}
        a = _lib.CompositeArgs()
        a.n_rays, a.n_samples, a.flags, a.distance_scale = n, s, flags, 1.0
        a.sigma, a.rgb, a.z = ins['sigma'].data_ptr(), ins['rgb'].data_ptr(), ins['z'].data_ptr()
        a.rays_d, a.rays_o, a.rays_d_ndc = d_dev.data_ptr(), o_dev.data_ptr(), dn.data_ptr()
        for k in ('rgb_map', 'acc', 'depth', 'depth_var', 'depth_ndc', 'depth_var_ndc', 'alpha', 'visibility',
                  'weights', 'd_sigma', 'd_rgb'):
            setattr(a, k, outs[k].data_ptr())
        a.g_rgb, a.g_acc, a.g_depth = gd['rgb'].data_ptr(), gd['acc'].data_ptr(), gd['depth'].data_ptr()
        a.g_depth_var, a.g_weights = gd['depth_var'].data_ptr(), gd['weights'].data_ptr()
        lib = _lib.load()
        st = _stream()
        if (flags & 4) and s > 256:
            return None
        _lib.check(lib.srf_composite_forward(ctypes.byref(a), st), 'forward')
        _lib.check(lib.srf_composite_backward(ctypes.byref(a), st), 'backward')
        torch.cuda.synchronize()
        del keep
        return {k: v.cpu() for k, v in outs.items()}

    staged, plain = run(False), run(True)
    for k in staged:
        scale = float(plain[k].abs().max()) if plain[k].numel() else 0.0
        torch.testing.assert_close(staged[k], plain[k], rtol=1e-5, atol=1e-6 * max(scale, 1e-30), msg=k)
    import ctypes as _c
    fl = _c.c_int(0)
    _lib_mod = __import__('simple_rf_gb300._lib', fromlist=['check'])
    _lib_mod.check(_lib_mod.load().srf_read_device_flag(_c.byref(fl), None), 'flag')
    assert fl.value == 0
