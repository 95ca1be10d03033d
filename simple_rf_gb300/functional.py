"""Torch-facing operators over the srf_gb300 C ABI.

Each operator allocates its outputs (and any workspace) with torch's caching
allocator, passes raw device pointers and the current CUDA stream to the C ABI,
and raises ``RuntimeError`` on a non-zero status.  Differentiable operators are
``torch.autograd.Function``s whose backward calls the hand-written adjoint
kernels.  Inputs must be contiguous float32 CUDA tensors; nothing here runs on
the CPU.
"""
import ctypes
import math

import torch

from . import _lib
from ._lib import call

class nvtx_range:
    """An NVTX range around one stage of a step (visible in profilers' timelines;
    under CUDA-graph capture it marks the capture, not the replays)."""

    def __init__(self, name):
        self.name = name

    def __enter__(self):
        torch.cuda.nvtx.range_push(self.name)
        return self

    def __exit__(self, *exc):
        torch.cuda.nvtx.range_pop()


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream(t=None):
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _require(t, name, shape=None, dtype=torch.float32):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f'{name} must be a tensor')
    if not t.is_cuda:
        raise RuntimeError(f'{name} must be a CUDA tensor (the srf_gb300 kernels have no CPU path)')
    if t.dtype != dtype:
        raise TypeError(f'{name} must be {dtype}, got {t.dtype}')
    if not t.is_contiguous():
        raise RuntimeError(f'{name} must be contiguous')
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise RuntimeError(f'{name} has shape {tuple(t.shape)}, expected {tuple(shape)}')
    return t


# ---------------------------------------------------------------- sampling --

def stratified_z(n_rays, n_samples, near, far, u=None, lindisp=False, device='cuda'):
    """SimpleNeRF17.py:330-358 (u: (N,S) uniforms, None = no jitter)."""
    z = torch.empty(n_rays, n_samples, device=device)
    if u is not None:
        _require(u, 'u', (n_rays, n_samples))
    call('srf_stratified_z', _ptr(z), _ptr(u), n_rays, n_samples, float(near), float(far), int(lindisp), _stream())
    return z


def sample_pdf(bins, weights, n_samples, u=None):
    """SimpleNeRF17.py:384-417."""
    n, nb = bins.shape
    _require(bins, 'bins')
    _require(weights, 'weights', (n, nb - 1))
    if u is not None:
        _require(u, 'u', (n, n_samples))
    out = torch.empty(n, n_samples, device=bins.device)
    if n:
        call('srf_sample_pdf', _ptr(out), _ptr(bins), _ptr(weights), _ptr(u), n, nb, n_samples, _stream())
    return out


def fine_z(z_coarse, weights_coarse, n_fine, u=None):
    """SimpleNeRF17.py:360-371: sorted [z_coarse, pdf samples] (no gradient)."""
    n, nc = z_coarse.shape
    _require(z_coarse, 'z_coarse')
    weights_coarse = weights_coarse.detach().contiguous()
    _require(weights_coarse, 'weights_coarse', (n, nc))
    if u is not None:
        _require(u, 'u', (n, n_fine))
    out = torch.empty(n, nc + n_fine, device=z_coarse.device)
    if n:  # an empty batch has NULL data pointers: nothing to launch
        call('srf_fine_z', _ptr(out), _ptr(z_coarse), _ptr(weights_coarse), _ptr(u), n, nc, n_fine, _stream())
    return out


def aabb_z(rays_o, rays_d, n_samples, bbox, near, far, step_size, u=None):
    """SimpleTensoRF09.py:388-400."""
    n = rays_o.shape[0]
    _require(rays_o, 'rays_o', (n, 3))
    _require(rays_d, 'rays_d', (n, 3))
    if u is not None:
        u = u.reshape(n).contiguous()
        _require(u, 'u', (n,))
    z = torch.empty(n, n_samples, device=rays_o.device)
    bb = _lib.host_floats([float(v) for v in torch.as_tensor(bbox).reshape(-1).tolist()])
    call('srf_aabb_z', _ptr(z), _ptr(rays_o), _ptr(rays_d), _ptr(u), n, n_samples, bb, float(near), float(far),
         float(step_size), _stream())
    return z


def ndc_rays(rays_o, rays_d, fx, fy, height, width, near):
    """CommonUtils04.py:120-149: NDC rays and view directions."""
    n = rays_o.shape[0]
    _require(rays_o, 'rays_o', (n, 3))
    _require(rays_d, 'rays_d', (n, 3))
    _require(fx, 'fx', (n,))
    _require(fy, 'fy', (n,))
    o = torch.empty_like(rays_o)
    d = torch.empty_like(rays_d)
    call('srf_ndc_rays', _ptr(rays_o), _ptr(rays_d), _ptr(fx), _ptr(fy), n, int(height), int(width), float(near),
         _ptr(o), _ptr(d), None, _stream())
    return o, d


def view_dirs(rays_d):
    """CommonUtils04.py:147-149."""
    n = rays_d.shape[0]
    _require(rays_d, 'rays_d', (n, 3))
    out = torch.empty_like(rays_d)
    call('srf_ndc_rays', None, _ptr(rays_d), None, None, n, 1, 1, 0.0, None, None, _ptr(out), _stream())
    return out


def positional_encoding(x, degree):
    """SimpleNeRF17.py:581-613 on (M, dims) rows."""
    m, dims = x.shape
    _require(x, 'x')
    out = torch.empty(m, dims * (2 * degree + 1), device=x.device)
    call('srf_positional_encoding', _ptr(out), out.shape[1], _ptr(x), m, dims, degree, _stream())
    return out


# ---------------------------------------------------------------- NeRF MLP --

class MlpSpec:
    """C descriptor of one reference MLP plus its parameter order."""

    def __init__(self, points_net_depth=8, points_net_width=256, views_net_depth=1, views_net_width=128,
                 points_pe_degree=10, views_pe_degree=4, use_view_dirs=True, view_dependent_rgb=True,
                 points_sigma_pe_degree=None, skip_layer=4):
        self.desc = _lib.NerfMlpDesc(points_net_depth, points_net_width, views_net_depth, views_net_width,
                                     points_pe_degree, views_pe_degree,
                                     -1 if points_sigma_pe_degree is None else points_sigma_pe_degree,
                                     int(use_view_dirs), int(view_dependent_rgb), skip_layer)
        self.use_view_dirs = bool(use_view_dirs)
        lib = _lib.load()
        n = lib.srf_nerf_mlp_num_params(ctypes.byref(self.desc))
        if n <= 0:
            raise RuntimeError('invalid MLP descriptor')
        self.param_names = []
        self.param_numel = []
        buf = ctypes.create_string_buffer(128)
        numel = ctypes.c_int64()
        for i in range(n):
            _lib.check(lib.srf_nerf_mlp_param_info(ctypes.byref(self.desc), i, buf, 128, ctypes.byref(numel)),
                       'srf_nerf_mlp_param_info')
            self.param_names.append(buf.value.decode())
            self.param_numel.append(numel.value)

    @classmethod
    def from_config(cls, c):
        """From a reference MLP config dict (NerfLlffTrainerTester10.py:296-370 form)."""
        if c.get('predict_visibility', False):
            raise NotImplementedError('predict_visibility is not supported by the srf_gb300 MLP')
        return cls(c['points_net_depth'], c['points_net_width'], c['views_net_depth'], c['views_net_width'],
                   c['points_positional_encoding_degree'], c.get('views_positional_encoding_degree', 0),
                   c['use_view_dirs'], c['view_dependent_rgb'], c.get('points_sigma_positional_encoding_degree'))

    def workspace_bytes(self, m, precision, for_backward):
        lib = _lib.load()
        return lib.srf_nerf_mlp_workspace_size(ctypes.byref(self.desc), m, precision, int(for_backward))


def _ptr_array(tensors):
    arr = (ctypes.c_void_p * len(tensors))()
    for i, t in enumerate(tensors):
        arr[i] = t.data_ptr()
    return arr


def loss_scaler(device, init_scale=65536.0):
    """A device srf_loss_scaler {scale, 1/scale, found_inf, growth_tracker} as a 16-byte tensor."""
    t = torch.empty(4, dtype=torch.float32, device=device)
    call('srf_loss_scaler_init', _ptr(t), float(init_scale), _stream())
    return t


def found_inf_ptr(scaler):
    """Device address of the scaler's found_inf word."""
    return None if scaler is None else ctypes.c_void_p(scaler.data_ptr() + 8)


# Bytes of saved activations one NerfMlpFunction call may hold between its
# forward and backward; None = half of the device memory free at the call.
_activation_budget = [None]


class activation_budget:
    """Context manager (or plain call) setting the activation budget of the
    NeRF MLP autograd op: ``with activation_budget(8 << 30): loss = model(...)``.

    A forward whose backward workspace would exceed the budget keeps only its
    inputs; its backward recomputes the activations ray chunk by ray chunk (each
    chunk within the budget) and accumulates the parameter gradients chunk by
    chunk.  ``None`` restores the default (half of the free device memory)."""

    def __init__(self, nbytes):
        self.prev = _activation_budget[0]
        _activation_budget[0] = None if nbytes is None else int(nbytes)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        _activation_budget[0] = self.prev


def recompute_rows(m, dir_div, budget, ws_bytes):
    """Rows per recomputation chunk: the largest multiple of lcm(dir_div, 128)
    (whole rays, and 512-byte aligned sub-tensor offsets) whose backward
    workspace ``ws_bytes(rows)`` fits ``budget``; 0 when all m rows fit (no
    recomputation).  Raises when even one unit exceeds the budget."""
    if m == 0 or ws_bytes(m) <= budget:
        return 0
    unit = dir_div * 128 // math.gcd(dir_div, 128)
    if ws_bytes(unit) > budget:
        raise RuntimeError(f'activation budget {budget} B is below one chunk of {unit} samples '
                           f'({ws_bytes(unit)} B of workspace)')
    lo, hi = 1, max(1, -(-m // unit))
    while lo < hi:  # largest k with ws_bytes(k * unit) <= budget
        mid = (lo + hi + 1) // 2
        if ws_bytes(mid * unit) <= budget:
            lo = mid
        else:
            hi = mid - 1
    return lo * unit


class NerfMlpFunction(torch.autograd.Function):
    """MLP.forward (SimpleNeRF17.py:696-785) with the hand-written backward.

    With SRF_PRECISION_FP16 each backward fits its own loss scale to the incoming
    gradients (the largest maps to about 2^10, leaving 2^5 of headroom for growth
    through the layers; srf_loss_scaler_fit); a gradient that still leaves the
    FP16 range gives non-finite parameter gradients and sets the scaler's
    found_inf.  The fused training step (train_step.py) instead carries one
    dynamic scale across steps and skips steps that overflow.

    When the activations the backward needs exceed the activation budget
    (:class:`activation_budget`), the forward runs chunk by chunk without keeping
    them and the backward recomputes each chunk's activations just before that
    chunk's adjoint (same kernels, same rows: the recomputed activations equal
    the first pass's bit for bit); the parameter gradients then sum the chunks'
    contributions (the order of the sum over samples differs from the unchunked
    pass by rounding only)."""

    @staticmethod
    def forward(ctx, spec, precision, pts, dirs, dir_div, noise, *params):
        m = pts.shape[0]
        _require(pts, 'pts', (m, 3))
        if spec.use_view_dirs:
            _require(dirs, 'dirs')
        if noise is not None:
            _require(noise, 'noise', (m,))
        params = [p.detach().contiguous() for p in params]
        need_grad = any(ctx.needs_input_grad[6:])
        sigma = torch.empty(m, device=pts.device)
        rgb = torch.empty(m, 3, device=pts.device)
        scaler = None
        if precision == _lib.SRF_PRECISION_FP16:
            scaler = loss_scaler(pts.device)
        rows = 0
        if need_grad:
            budget = _activation_budget[0]
            if budget is None:
                budget = torch.cuda.mem_get_info(pts.device)[0] // 2
            rows = recompute_rows(m, dir_div, budget, lambda r: spec.workspace_bytes(r, precision, True))
        ctx.spec, ctx.precision, ctx.dir_div, ctx.m, ctx.scaler = spec, precision, dir_div, m, scaler
        ctx.params = params
        ctx.rows = rows
        ctx.set_materialize_grads(True)
        if m == 0:  # an empty batch has NULL data pointers: nothing to launch
            ctx.ws = None
            return sigma, rgb
        if rows:
            ws = torch.empty(max(spec.workspace_bytes(rows, precision, False), 1), dtype=torch.uint8,
                             device=pts.device)
            for r0 in range(0, m, rows):
                _mlp_chunk_forward(spec, precision, params, pts, dirs, dir_div, noise, r0, min(rows, m - r0),
                                   sigma, rgb, False, ws, scaler)
            ctx.inputs = (pts, dirs, noise)
            ctx.ws = None
            return sigma, rgb
        ws = torch.empty(max(spec.workspace_bytes(m, precision, need_grad), 1), dtype=torch.uint8,
                         device=pts.device)
        call('srf_nerf_mlp_forward', ctypes.byref(spec.desc), _ptr_array(params), _ptr(pts), _ptr(dirs),
             int(dir_div), m, _ptr(noise), _ptr(sigma), _ptr(rgb), precision, int(need_grad), _ptr(ws),
             ws.numel(), _ptr(scaler), _stream())
        ctx.ws = ws if need_grad else None
        return sigma, rgb

    @staticmethod
    def backward(ctx, dsigma, drgb):
        if ctx.m == 0:
            return (None, None, None, None, None, None) + tuple(torch.zeros_like(p) for p in ctx.params)
        grads = [torch.empty_like(p) for p in ctx.params]
        dsigma = dsigma.contiguous()
        drgb = drgb.contiguous()
        if ctx.scaler is not None:
            call('srf_loss_scaler_fit', _ptr(ctx.scaler), _ptr(dsigma), dsigma.numel(), _ptr(drgb), drgb.numel(),
                 1024.0, _stream())
        if ctx.rows:
            spec, precision, m, rows = ctx.spec, ctx.precision, ctx.m, ctx.rows
            pts, dirs, noise = ctx.inputs
            dev = pts.device
            ws = torch.empty(max(spec.workspace_bytes(rows, precision, True), 1), dtype=torch.uint8, device=dev)
            sig = torch.empty(rows, device=dev)
            col = torch.empty(rows, 3, device=dev)
            gp = _ptr_array(grads)
            for i, r0 in enumerate(range(0, m, rows)):
                r = min(rows, m - r0)
                _mlp_chunk_forward(spec, precision, ctx.params, pts, dirs, ctx.dir_div, noise, r0, r, sig, col,
                                   True, ws, ctx.scaler, out_offset=False)
                call('srf_nerf_mlp_backward', ctypes.byref(spec.desc), _ptr_array(ctx.params),
                     _ptr_at(dsigma, r0), _ptr_at(drgb, 3 * r0), int(ctx.dir_div), r, gp, int(i > 0), precision,
                     _ptr(ws), ws.numel(), _ptr(ctx.scaler), _stream())
            ctx.inputs = None
            return (None, None, None, None, None, None) + tuple(grads)
        call('srf_nerf_mlp_backward', ctypes.byref(ctx.spec.desc), _ptr_array(ctx.params), _ptr(dsigma), _ptr(drgb),
             int(ctx.dir_div), ctx.m, _ptr_array(grads), 0, ctx.precision, _ptr(ctx.ws), ctx.ws.numel(),
             _ptr(ctx.scaler), _stream())
        ctx.ws = None
        return (None, None, None, None, None, None) + tuple(grads)


def _ptr_at(t, offset):
    """Device address of element ``offset`` of a contiguous tensor (None passes through)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr() + offset * t.element_size())


def _mlp_chunk_forward(spec, precision, params, pts, dirs, dir_div, noise, r0, r, sigma, rgb, for_backward, ws,
                       scaler, out_offset=True):
    """srf_nerf_mlp_forward over rows [r0, r0 + r) (r0 a multiple of dir_div);
    outputs at the same rows of sigma/rgb, or at their start with out_offset=False."""
    o = r0 if out_offset else 0
    call('srf_nerf_mlp_forward', ctypes.byref(spec.desc), _ptr_array(params), _ptr_at(pts, 3 * r0),
         _ptr_at(dirs, 3 * (r0 // dir_div)), int(dir_div), r, _ptr_at(noise, r0), _ptr_at(sigma, o),
         _ptr_at(rgb, 3 * o), precision, int(for_backward), _ptr(ws), ws.numel(), _ptr(scaler), _stream())


# -------------------------------------------------------------- compositing --

_COMPOSITE_OUT = ('rgb', 'acc', 'depth', 'depth_var', 'alpha', 'visibility', 'weights', 'depth_ndc', 'depth_var_ndc')


class CompositeFunction(torch.autograd.Function):
    """volume_rendering (SimpleNeRF17.py:486-539) / get_volume_rendering_weights +
    volume_render (SimpleTensoRF09.py:767-819); the adjoint is a reverse scan."""

    @staticmethod
    def forward(ctx, sigma, rgb, z, rays_d, rays_o, rays_d_ndc, flags, distance_scale, white_per_ray):
        n, s = sigma.shape
        _require(sigma, 'sigma', (n, s))
        if rgb is not None:
            _require(rgb, 'rgb', (n, s, 3))
        _require(z, 'z', (n, s))
        _require(rays_d, 'rays_d', (n, 3))
        ndc = bool(flags & _lib.SRF_COMPOSITE_NDC)
        dev = sigma.device
        out = dict.fromkeys(_COMPOSITE_OUT)
        out['rgb'] = torch.empty(n, 3, device=dev)
        for k in ('acc', 'depth', 'depth_var'):
            out[k] = torch.empty(n, device=dev)
        for k in ('alpha', 'visibility', 'weights'):
            out[k] = torch.empty(n, s, device=dev)
        if ndc:
            out['depth_ndc'] = torch.empty(n, device=dev)
            out['depth_var_ndc'] = torch.empty(n, device=dev)
        a = _lib.CompositeArgs()
        a.n_rays, a.n_samples, a.flags, a.distance_scale = n, s, int(flags), float(distance_scale)
        a.sigma, a.rgb, a.z, a.rays_d = sigma.data_ptr(), _ptr(rgb), z.data_ptr(), rays_d.data_ptr()
        if ndc:
            a.rays_o, a.rays_d_ndc = rays_o.data_ptr(), rays_d_ndc.data_ptr()
        if white_per_ray is not None:
            a.white_per_ray = white_per_ray.data_ptr()
        for k in _COMPOSITE_OUT:
            if out[k] is not None:
                setattr(a, 'rgb_map' if k == 'rgb' else k, out[k].data_ptr())
        if n:
            call('srf_composite_forward', ctypes.byref(a), _stream())
        ctx.save_for_backward(sigma, rgb, z, rays_d, rays_o, rays_d_ndc, white_per_ray)
        ctx.flags, ctx.ds = int(flags), float(distance_scale)
        ctx.set_materialize_grads(False)
        return tuple(out[k] if out[k] is not None else torch.empty(0, device=dev) for k in _COMPOSITE_OUT)

    @staticmethod
    def backward(ctx, g_rgb, g_acc, g_depth, g_depth_var, g_alpha, g_vis, g_weights, g_depth_ndc, g_depth_var_ndc):
        sigma, rgb, z, rays_d, rays_o, rays_d_ndc, white = ctx.saved_tensors
        if (g_alpha is not None and bool(g_alpha.any())) or (g_vis is not None and bool(g_vis.any())):
            raise NotImplementedError('gradients through alpha/visibility outputs are not supported')
        n, s = sigma.shape
        a = _lib.CompositeArgs()
        a.n_rays, a.n_samples, a.flags, a.distance_scale = n, s, ctx.flags, ctx.ds
        a.sigma, a.rgb, a.z, a.rays_d = sigma.data_ptr(), _ptr(rgb), z.data_ptr(), rays_d.data_ptr()
        if ctx.flags & _lib.SRF_COMPOSITE_NDC:
            a.rays_o, a.rays_d_ndc = rays_o.data_ptr(), rays_d_ndc.data_ptr()
        if white is not None:
            a.white_per_ray = white.data_ptr()
        keep = []
        for name, g in (('g_rgb', g_rgb), ('g_acc', g_acc), ('g_depth', g_depth), ('g_depth_var', g_depth_var),
                        ('g_weights', g_weights), ('g_depth_ndc', g_depth_ndc),
                        ('g_depth_var_ndc', g_depth_var_ndc)):
            if g is not None and g.numel() > 0:
                g = g.contiguous()
                keep.append(g)
                setattr(a, name, g.data_ptr())
        d_sigma = torch.empty_like(sigma)
        d_rgb = torch.empty_like(rgb) if rgb is not None and ctx.needs_input_grad[1] else None
        a.d_sigma, a.d_rgb = d_sigma.data_ptr(), _ptr(d_rgb)
        if n:
            call('srf_composite_backward', ctypes.byref(a), _stream())
        return d_sigma, d_rgb, None, None, None, None, None, None, None


def adam_step(param, grad, exp_avg, exp_avg_sq, *, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0, step):
    """In-place fused Adam update (torch.optim.Adam semantics)."""
    for name, x in (('param', param), ('grad', grad), ('exp_avg', exp_avg), ('exp_avg_sq', exp_avg_sq)):
        _require(x, name, param.shape)
    call('srf_adam_step', _ptr(param), _ptr(grad), _ptr(exp_avg), _ptr(exp_avg_sq), param.numel(), float(lr),
         float(beta1), float(beta2), float(eps), float(weight_decay), int(step), None, None, _stream())


def _dense(t):
    return t.is_contiguous() or (t.dim() == 4 and t.is_contiguous(memory_format=torch.channels_last))


def adam_multi_step(tensors, *, step, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0, step_dev=None,
                    skip_dev=None):
    """In-place Adam over ``tensors`` = [(param, grad, exp_avg, exp_avg_sq, lr), ...]
    with one launch per 64 tensors (each tensor's four buffers share one dense layout).
    ``step_dev`` (device int32, read instead of ``step``) and ``skip_dev`` (device
    int32: nonzero skips the update) keep the step free of host values, for
    graph capture."""
    arr = (_lib.AdamTensor * len(tensors))()
    for i, (p, g, m, v, lr) in enumerate(tensors):
        for name, x in (('param', p), ('grad', g), ('exp_avg', m), ('exp_avg_sq', v)):
            if not x.is_cuda or x.dtype != torch.float32:
                raise RuntimeError(f'tensor {i} {name} must be a float32 CUDA tensor')
            if x.shape != p.shape or x.stride() != p.stride() or not _dense(x):
                raise RuntimeError(f'tensor {i} {name}: layout {tuple(x.shape)} {x.stride()} does not match the '
                                   f'dense param {tuple(p.shape)} {p.stride()}')
        arr[i] = _lib.AdamTensor(p.data_ptr(), g.data_ptr(), m.data_ptr(), v.data_ptr(), p.numel(), float(lr))
    call('srf_adam_multi_step', arr, len(tensors), float(beta1), float(beta2), float(eps), float(weight_decay),
         int(step), _ptr(step_dev), _ptr(skip_dev), _stream())


def rgb_depth_loss(rgb, target_rgb, depth, target_depth, depth_mask, n_depth_rays, depth_weight, loss=None):
    """Loss of one net's outputs and its gradients w.r.t. rgb (N,3) and depth (N,)."""
    n = rgb.shape[0]
    if loss is None:
        loss = torch.zeros(1, device=rgb.device)
    g_rgb = torch.empty_like(rgb)
    g_depth = torch.empty_like(depth)
    call('srf_rgb_depth_loss', _ptr(rgb), _ptr(target_rgb), _ptr(depth), _ptr(target_depth), _ptr(depth_mask), n,
         int(n_depth_rays), float(depth_weight), _ptr(loss), _ptr(g_rgb), _ptr(g_depth), _stream())
    return loss, g_rgb, g_depth


def composite(sigma, rgb, z, rays_d, *, ndc=False, rays_o=None, rays_d_ndc=None, white_bkgd=False,
              distance_scale=1.0, white_per_ray=None):
    """Returns the reference's volume-rendering dict (keys as SimpleNeRF17.py:521-533)."""
    flags = (_lib.SRF_COMPOSITE_NDC if ndc else 0) | (_lib.SRF_COMPOSITE_WHITE_BKGD if white_bkgd else 0)
    if white_per_ray is not None:
        white_per_ray = white_per_ray.to(torch.uint8).contiguous()
    outs = CompositeFunction.apply(sigma.contiguous(), None if rgb is None else rgb.contiguous(), z.contiguous(),
                                   rays_d.contiguous(),
                                   None if rays_o is None else rays_o.contiguous(),
                                   None if rays_d_ndc is None else rays_d_ndc.contiguous(), flags, distance_scale,
                                   white_per_ray)
    d = dict(zip(_COMPOSITE_OUT, outs))
    if not ndc:
        del d['depth_ndc'], d['depth_var_ndc']
    return d


def pixel_rays(pixel_id, intrinsics, extrinsics, half_pixel=False):
    """CommonUtils04.py:73-95 get_rays_tr: world rays of (image, x, y) pixel ids."""
    n = pixel_id.shape[0]
    pid = pixel_id.to(torch.int32).contiguous()
    k = intrinsics.float().contiguous()
    e = extrinsics.float().contiguous()
    _require(k, 'intrinsics', (n, 3, 3))
    _require(e, 'extrinsics', (n, 4, 4))
    o = torch.empty(n, 3, device=k.device)
    d = torch.empty(n, 3, device=k.device)
    call('srf_pixel_rays', _ptr(pid), _ptr(k), _ptr(e), n, int(half_pixel), _ptr(o), _ptr(d), _stream())
    return o, d


_TV_MAX = 8


def _tv_struct(comps, grads=None):
    arr = (_lib.TvComponent * len(comps))()
    for i, p in enumerate(comps):
        if p.dim() != 4 or p.shape[0] != 1:
            raise ValueError(f'TV component {i}: expected (1, R, H, W), got {tuple(p.shape)}')
        if not p.is_cuda or p.dtype != torch.float32:
            raise RuntimeError(f'TV component {i} must be a float32 CUDA tensor (the srf_gb300 kernels have no '
                               'CPU path)')
        g = None if grads is None else grads[i]
        if g is not None and (g.stride() != p.stride() or g.shape != p.shape):
            raise ValueError(f'TV component {i}: gradient strides {g.stride()} differ from {p.stride()}')
        arr[i] = _lib.TvComponent(p.data_ptr(), None if g is None else g.data_ptr(), p.shape[1], p.shape[2],
                                  p.shape[3], p.stride(1), p.stride(2), p.stride(3))
    return arr


class TvLossFunction(torch.autograd.Function):
    """srf_tv_loss forward (loss only) and backward (gradients scaled by the incoming
    gradient on the device)."""

    @staticmethod
    def forward(ctx, weight, *comps):
        loss = torch.zeros((), device=comps[0].device)
        for i in range(0, len(comps), _TV_MAX):
            part = comps[i:i + _TV_MAX]
            call('srf_tv_loss', _tv_struct(part), len(part), float(weight), None, _ptr(loss), _stream())
        ctx.save_for_backward(*comps)
        ctx.weight = float(weight)
        return loss

    @staticmethod
    def backward(ctx, g):
        comps = ctx.saved_tensors
        grads = [torch.zeros_like(p) for p in comps]
        g = g.float().contiguous()
        for i in range(0, len(comps), _TV_MAX):
            part = comps[i:i + _TV_MAX]
            call('srf_tv_loss', _tv_struct(part, grads[i:i + _TV_MAX]), len(part), ctx.weight, _ptr(g), None,
                 _stream())
        return (None, *grads)


def tv_loss(components, weight=1.0):
    """weight * TotalVariationLoss04.compute_tv_loss's sum over (1, R, H, W) grids
    (src/loss_functions/TotalVariationLoss04.py:97-116), differentiable."""
    comps = [p if p.dtype == torch.float32 else p.float() for p in components]
    if not comps:
        return torch.zeros(())
    return TvLossFunction.apply(float(weight), *comps)


def tv_loss_accumulate(components, weight, loss=None):
    """The same loss added into ``loss`` (a device scalar, may be None) with each
    component's gradient added into its ``.grad`` in the same launch (for fused
    training steps that own the gradient buffers)."""
    comps = list(components)
    for p in comps:
        if p.grad is None:
            p.grad = torch.zeros_like(p)
    for i in range(0, len(comps), _TV_MAX):
        part = comps[i:i + _TV_MAX]
        call('srf_tv_loss', _tv_struct([p.detach() for p in part], [p.grad for p in part]), len(part),
             float(weight), None, _ptr(loss), _stream())
    return loss


class _DepthMseFunction(torch.autograd.Function):
    """mean over the masked rays of (pred - target)^2 with the target detached
    (srf_depth_mse_loss with mean_over_mask): SparseDepthMSE14.compute_depth_loss
    (src/loss_functions/SparseDepthMSE14.py:84-97) and CoarseFineConsistencyLoss34.compute_loss_sd
    (src/loss_functions/CoarseFineConsistencyLoss34.py:170-187)."""

    @staticmethod
    def forward(ctx, pred, target, mask):
        p = pred.detach().contiguous().float()
        t = target.detach().contiguous().float()
        m = mask.to(torch.uint8).contiguous()
        loss = torch.zeros(1, device=p.device)
        g = torch.zeros_like(p)
        call('srf_depth_mse_loss', _ptr(p), _ptr(t), _ptr(m), p.shape[0], 1.0, 1, _ptr(loss), _ptr(g), None,
             _stream())
        ctx.save_for_backward(g)
        return loss[0]

    @staticmethod
    def backward(ctx, g_loss):
        (g,) = ctx.saved_tensors
        return g * g_loss, None, None


def depth_mse(pred, target, mask):
    return _DepthMseFunction.apply(pred, target, mask)
