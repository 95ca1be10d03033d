"""Fused Simple-NeRF training step on one GPU, driven through the C ABI.

One step = Trainer10.train_one_iter (src/Trainer10.py:65-115) for a NeRF with a
coarse and a fine net, restated as a fixed sequence of hand-written kernels:

    view dirs -> stratified z (SimpleNeRF17.py:330-358) -> sample points ->
    coarse PE+MLP -> composite (:486-539) -> inverse-CDF fine z + merge sort
    (:360-417) -> fine PE+MLP -> composite -> loss (rgb MSE + weighted L1 depth
    on the depth-supervised rays) -> composite adjoints (reverse scans) ->
    MLP adjoints -> fused Adam on FP32 master weights.

Every buffer is allocated once, so the whole step can be captured as one CUDA
graph and replayed.  ``precision='bf16'`` runs the MLP GEMMs on tcgen05 tensor
cores (BF16 operands, FP32 accumulation); ``'fp32'`` is the plain path.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .functional import MlpSpec, _ptr_array

_P = ctypes.c_void_p


def _vp(t):
    return None if t is None else _P(t.data_ptr())


def xavier_uniform_(flat_views, spec, rng):
    """Xavier-uniform weights and zero biases (the init the benchmark configs name)."""
    for name, t in zip(spec.param_names, flat_views):
        if name.endswith('weight'):
            fan_out, fan_in = t.shape
            bound = np.sqrt(6.0 / (fan_in + fan_out))
            t.copy_(torch.from_numpy(rng.uniform(-bound, bound, size=tuple(t.shape)).astype(np.float32)))
        else:
            t.zero_()


class NetState:
    """FP32 master parameters, gradients and Adam moments of one MLP, as flat buffers."""

    def __init__(self, spec, device, rng=None):
        self.spec = spec
        shapes = list(zip(spec.param_names, spec.param_numel))
        total = sum(n for _, n in shapes)
        self.flat = torch.zeros(total, device=device)
        self.grad = torch.zeros(total, device=device)
        self.m = torch.zeros(total, device=device)
        self.v = torch.zeros(total, device=device)
        self.views, self.gviews = [], []
        off = 0
        for (name, numel), shape in zip(shapes, self._shapes(spec)):
            self.views.append(self.flat[off:off + numel].view(shape))
            self.gviews.append(self.grad[off:off + numel].view(shape))
            off += numel
        self.pptr = _ptr_array(self.views)
        self.gptr = _ptr_array(self.gviews)
        if rng is not None:
            with torch.no_grad():
                xavier_uniform_(self.views, spec, rng)

    @staticmethod
    def _shapes(spec):
        d = spec.desc
        shapes = []
        ppe = 3 * (2 * d.points_pe_degree + 1)
        pin = ppe if d.points_sigma_pe_degree < 0 else 3 * (2 * d.points_sigma_pe_degree + 1)
        vpe = 3 * (2 * d.views_pe_degree + 1) if d.use_view_dirs else 0
        vin = vpe + ppe - pin
        wp, wv = d.points_net_width, d.views_net_width
        for j in range(d.points_net_depth):
            k = pin if j == 0 else (wp + pin if j - 1 == d.skip_layer else wp)
            shapes += [(wp, k), (wp,)]
        if d.view_dependent_rgb:
            for j in range(d.views_net_depth):
                shapes += [(wv, vin + wp if j == 0 else wv), (wv,)]
        no = 1 if d.view_dependent_rgb else 4
        shapes += [(no, wp), (no,)]
        if d.view_dependent_rgb:
            shapes += [(wp, wp), (wp,), (3, wv), (3,)]
        return shapes

    def state_dict(self):
        return {n: v.detach().clone() for n, v in zip(self.spec.param_names, self.views)}


class NerfTrainStep:
    """Preallocated, graph-capturable config-2 training step (coarse + fine NeRF)."""

    def __init__(self, n_rays=4096, n_coarse=64, n_fine=128, near=2.0, far=6.0, white_bkgd=True,
                 depth_fraction=0.25, depth_weight=0.1, precision='bf16', spec_kwargs=None, lr=5e-4,
                 betas=(0.9, 0.999), eps=1e-8, seed=0, device='cuda'):
        self.dev = torch.device(device)
        self.n, self.sc, self.sf = n_rays, n_coarse, n_fine
        self.s = n_coarse + n_fine
        self.near, self.far = float(near), float(far)
        self.white = bool(white_bkgd)
        self.n_depth = max(int(round(n_rays * depth_fraction)), 0)
        self.depth_weight = float(depth_weight)
        self.precision = _lib.SRF_PRECISION_BF16 if precision == 'bf16' else _lib.SRF_PRECISION_FP32
        self.lr, self.betas, self.eps = float(lr), betas, float(eps)
        self.spec = MlpSpec(**(spec_kwargs or {}))
        rng = np.random.default_rng(seed)
        self.nets = {'coarse': NetState(self.spec, self.dev, rng), 'fine': NetState(self.spec, self.dev, rng)}
        n, sc, s = n_rays, n_coarse, self.s
        f32 = dict(device=self.dev, dtype=torch.float32)
        # inputs (static buffers the host copies into)
        self.rays_o = torch.zeros(n, 3, **f32)
        self.rays_d = torch.zeros(n, 3, **f32)
        self.target_rgb = torch.zeros(n, 3, **f32)
        self.target_depth = torch.zeros(n, **f32)
        self.u_c = torch.zeros(n, sc, **f32)
        self.u_f = torch.zeros(n, n_fine, **f32)
        self.depth_mask = torch.zeros(n, dtype=torch.uint8, device=self.dev)
        self.depth_mask[:self.n_depth] = 1
        # intermediates
        self.vdirs = torch.zeros(n, 3, **f32)
        self.buf = {}
        for tag, ss in (('coarse', sc), ('fine', s)):
            b = {'z': torch.zeros(n, ss, **f32), 'pts': torch.zeros(n * ss, 3, **f32), 'sigma': torch.zeros(n * ss, **f32),
                 'rgb': torch.zeros(n * ss, 3, **f32), 'rgb_map': torch.zeros(n, 3, **f32), 'acc': torch.zeros(n, **f32),
                 'depth': torch.zeros(n, **f32), 'depth_var': torch.zeros(n, **f32), 'weights': torch.zeros(n, ss, **f32),
                 'g_rgb': torch.zeros(n, 3, **f32), 'g_depth': torch.zeros(n, **f32),
                 'd_sigma': torch.zeros(n * ss, **f32), 'd_rgb': torch.zeros(n * ss, 3, **f32)}
            ws_bytes = self.spec.workspace_bytes(n * ss, self.precision, True)
            if ws_bytes == 0:
                raise RuntimeError('MLP configuration not supported at this precision')
            b['ws'] = torch.empty(ws_bytes, dtype=torch.uint8, device=self.dev)
            self.buf[tag] = b
        self.loss = torch.zeros(1, **f32)
        self.step_count = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.graph = None
        self.launches_per_step = None

    # ------------------------------------------------------------ enqueue --
    def _composite_args(self, tag, backward):
        b = self.buf[tag]
        ss = b['z'].shape[1]
        a = _lib.CompositeArgs()
        a.n_rays, a.n_samples = self.n, ss
        a.flags = _lib.SRF_COMPOSITE_WHITE_BKGD if self.white else 0
        a.distance_scale = 1.0
        a.sigma, a.rgb, a.z, a.rays_d = b['sigma'].data_ptr(), b['rgb'].data_ptr(), b['z'].data_ptr(), \
            self.rays_d.data_ptr()
        if not backward:
            a.rgb_map, a.acc, a.depth = b['rgb_map'].data_ptr(), b['acc'].data_ptr(), b['depth'].data_ptr()
            a.depth_var, a.weights = b['depth_var'].data_ptr(), b['weights'].data_ptr()
        else:
            a.g_rgb, a.g_depth = b['g_rgb'].data_ptr(), b['g_depth'].data_ptr()
            a.d_sigma, a.d_rgb = b['d_sigma'].data_ptr(), b['d_rgb'].data_ptr()
        return a

    def _enqueue(self):
        lib = _lib.load()
        st = _P(torch.cuda.current_stream(self.dev).cuda_stream)
        chk = _lib.check
        n = self.n
        chk(lib.srf_ndc_rays(None, _vp(self.rays_d), None, None, n, 1, 1, 0.0, None, None, _vp(self.vdirs), st),
            'view_dirs')
        self.loss.zero_()
        chk(lib.srf_stratified_z(_vp(self.buf['coarse']['z']), _vp(self.u_c), n, self.sc, self.near, self.far, 0, st),
            'stratified_z')
        for tag in ('coarse', 'fine'):
            b = self.buf[tag]
            net = self.nets[tag]
            ss = b['z'].shape[1]
            if tag == 'fine':
                cb = self.buf['coarse']
                chk(lib.srf_fine_z(_vp(b['z']), _vp(cb['z']), _vp(cb['weights']), _vp(self.u_f), n, self.sc, self.sf,
                                   st), 'fine_z')
            chk(lib.srf_ray_points(_vp(self.rays_o), _vp(self.rays_d), _vp(b['z']), n, ss, _vp(b['pts']), st),
                'ray_points')
            chk(lib.srf_nerf_mlp_forward(ctypes.byref(self.spec.desc), net.pptr, _vp(b['pts']), _vp(self.vdirs), ss,
                                         n * ss, None, _vp(b['sigma']), _vp(b['rgb']), self.precision, 1, _vp(b['ws']),
                                         b['ws'].numel(), st), 'mlp_forward')
            chk(lib.srf_composite_forward(ctypes.byref(self._composite_args(tag, False)), st), 'composite_forward')
            chk(lib.srf_rgb_depth_loss(_vp(b['rgb_map']), _vp(self.target_rgb), _vp(b['depth']),
                                       _vp(self.target_depth), _vp(self.depth_mask), n, self.n_depth,
                                       self.depth_weight, _vp(self.loss), _vp(b['g_rgb']), _vp(b['g_depth']), st),
                'loss')
        for tag in ('fine', 'coarse'):
            b = self.buf[tag]
            net = self.nets[tag]
            ss = b['z'].shape[1]
            chk(lib.srf_composite_backward(ctypes.byref(self._composite_args(tag, True)), st), 'composite_backward')
            chk(lib.srf_nerf_mlp_backward(ctypes.byref(self.spec.desc), net.pptr, _vp(b['d_sigma']), _vp(b['d_rgb']),
                                          ss, n * ss, net.gptr, 0, self.precision, _vp(b['ws']), b['ws'].numel(), st),
                'mlp_backward')
        chk(lib.srf_counter_add(_vp(self.step_count), 1, st), 'counter')
        for net in self.nets.values():
            chk(lib.srf_adam_step(_vp(net.flat), _vp(net.grad), _vp(net.m), _vp(net.v), net.flat.numel(), self.lr,
                                  self.betas[0], self.betas[1], self.eps, 0.0, 1, _vp(self.step_count), st), 'adam')

    # ------------------------------------------------------------- public --
    def set_batch(self, rays_o, rays_d, target_rgb, target_depth, u_coarse, u_fine, non_blocking=True):
        """Copy one batch (host pinned or device tensors) into the step's input buffers."""
        for dst, src in ((self.rays_o, rays_o), (self.rays_d, rays_d), (self.target_rgb, target_rgb),
                         (self.target_depth, target_depth), (self.u_c, u_coarse), (self.u_f, u_fine)):
            dst.copy_(src, non_blocking=non_blocking)

    def capture(self, warmup=2):
        """Run ``warmup`` eager steps (sets kernel attributes, fills allocator pools),
        then capture one step as a CUDA graph."""
        s = torch.cuda.Stream(self.dev)
        s.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(s):
            for _ in range(warmup):
                self._enqueue()
        torch.cuda.current_stream(self.dev).wait_stream(s)
        torch.cuda.synchronize(self.dev)
        lib = _lib.load()
        before = lib.srf_launch_count()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._enqueue()
        self.launches_per_step = int(lib.srf_launch_count() - before)
        torch.cuda.synchronize(self.dev)

    def step(self):
        """Enqueue one training step on the current stream (graph replay when captured)."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self._enqueue()

    def outputs(self):
        return {f'{k}_{tag}': self.buf[tag][k] for tag in ('coarse', 'fine')
                for k in ('rgb_map', 'acc', 'depth', 'depth_var', 'weights', 'z')}


def main(argv=None):
    """Run the fused training step on synthetic config-2 data and print ms/step:

        python -m simple_rf_gb300.train_step --rays 4096 --steps 10 --warmup 3 [--precision fp32] [--eager]
    """
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument('--rays', type=int, default=4096)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--precision', default='bf16', choices=['bf16', 'fp32'])
    ap.add_argument('--eager', action='store_true', help='launch kernels directly instead of replaying a CUDA graph')
    args = ap.parse_args(argv)
    from . import build as _build
    _build.build()
    dev = torch.device('cuda')
    step = NerfTrainStep(args.rays, 64, 128, precision=args.precision, device=dev)
    step.set_batch(*synthetic_batch(args.rays, 64, 128, seed=1, device=dev))
    if not args.eager:
        step.capture(warmup=1)
    for _ in range(args.warmup):
        step.step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step.step()
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / max(args.steps, 1)
    print(json.dumps({'rays': args.rays, 'precision': args.precision, 'graph': not args.eager,
                      'ms_per_step': round(ms, 4), 'rays_per_s': round(args.rays / ms * 1e3, 1),
                      'loss': float(step.loss.item())}))


def synthetic_batch(n_rays, n_coarse, n_fine, seed, device='cpu', pin=False):
    """Config-2 synthetic inputs: o ~ N(0, 0.1^2), d = normalize(N(0, I)), rgb
    targets ~ U[0,1]^3, depth targets ~ U[2,6], stratified/pdf uniforms ~ U[0,1)."""
    g = torch.Generator().manual_seed(seed)
    o = torch.randn(n_rays, 3, generator=g) * 0.1
    d = torch.randn(n_rays, 3, generator=g)
    d = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    t_rgb = torch.rand(n_rays, 3, generator=g)
    t_depth = torch.rand(n_rays, generator=g) * 4 + 2
    u_c = torch.rand(n_rays, n_coarse, generator=g)
    u_f = torch.rand(n_rays, n_fine, generator=g)
    out = [o, d, t_rgb, t_depth, u_c, u_f]
    if pin:
        out = [x.pin_memory() for x in out]
    if str(device) != 'cpu':
        out = [x.to(device) for x in out]
    return out


if __name__ == '__main__':
    main()
