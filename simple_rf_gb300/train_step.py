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
cores (BF16 operands, FP32 accumulation); ``'fp16'`` does the same with FP16
operands and a dynamic loss scale (GradScaler semantics, kept on the device: a
step whose scaled gradients overflow is skipped and halves the scale); ``'fp32'``
is the plain path.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from . import functional as F
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


class _Net:
    """One MLP evaluated in the step: its parameters and its per-sample buffers."""

    def __init__(self, name, level, spec, state, n, ss, precision, dev, train=True):
        f32 = dict(device=dev, dtype=torch.float32)
        self.name, self.level, self.spec, self.state = name, level, spec, state
        self.b = {'sigma': torch.zeros(n * ss, **f32), 'rgb': torch.zeros(n * ss, 3, **f32),
                  'rgb_map': torch.zeros(n, 3, **f32), 'acc': torch.zeros(n, **f32), 'depth': torch.zeros(n, **f32),
                  'depth_var': torch.zeros(n, **f32), 'weights': torch.zeros(n, ss, **f32),
                  'depth_ndc': torch.zeros(n, **f32), 'depth_var_ndc': torch.zeros(n, **f32),
                  'g_rgb': torch.zeros(n, 3, **f32), 'g_depth': torch.zeros(n, **f32),
                  'd_sigma': torch.zeros(n * ss, **f32), 'd_rgb': torch.zeros(n * ss, 3, **f32)}
        if not train:
            for k in ('g_rgb', 'g_depth', 'd_sigma', 'd_rgb'):
                del self.b[k]
        ws_bytes = spec.workspace_bytes(n * ss, precision, train)
        if ws_bytes == 0:
            raise RuntimeError(f'MLP configuration of {name} not supported at this precision')
        self.b['ws'] = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)


class NerfTrainStep:
    """Preallocated, graph-capturable Simple-NeRF training step.

    The 4096-ray training form (default): world rays, coarse + fine nets, white background.
    The NDC pair form: ``ndc=dict(h=378, w=504, focal=400.0, near=1.0)`` switches to
    forward-facing NDC rays (CommonUtils04.py:120-138; z in [near_ndc, far_ndc] =
    [0, 1]) and ``aug=[(name, spec_kwargs), ...]`` adds augmented nets evaluated
    on the same coarse samples (SimpleNeRF17.py:244-261) and, with
    ``aug_fine=True``, on the fine samples too (:296-313).  Each augmented net is
    trained on the rgb loss, and its (detached) coarse depth is a squared-error
    target of the main coarse depth with ``consistency_weight``
    (AugmentationsDepthLoss11.py:208-226 with every ray trusting the augmented net).
    """

    def __init__(self, n_rays=4096, n_coarse=64, n_fine=128, near=2.0, far=6.0, white_bkgd=True,
                 depth_fraction=0.25, depth_weight=0.1, precision='bf16', spec_kwargs=None, lr=5e-4,
                 betas=(0.9, 0.999), eps=1e-8, seed=0, device='cuda', ndc=None, aug=None, aug_fine=False,
                 consistency_weight=0.1, train=True, perturb=True, loss_scale_init=65536.0, concurrent_aug=True,
                 overlap_coarse=True):
        self.dev = torch.device(device)
        self.n, self.sc, self.sf = n_rays, n_coarse, n_fine
        self.s = n_coarse + n_fine
        self.ndc = dict(ndc) if ndc else None
        self.near, self.far = (0.0, 1.0) if self.ndc else (float(near), float(far))
        self.white = bool(white_bkgd)
        self.n_depth = max(int(round(n_rays * depth_fraction)), 0)
        self.depth_weight = float(depth_weight)
        self.consistency_weight = float(consistency_weight)
        self.train, self.perturb = bool(train), bool(perturb)
        self.precision = _lib.PRECISIONS[precision]
        self.scaler = F.loss_scaler(self.dev, loss_scale_init) if self.precision == _lib.SRF_PRECISION_FP16 else None
        self.found_inf = F.found_inf_ptr(self.scaler)
        self.lr, self.betas, self.eps = float(lr), betas, float(eps)
        self.spec = MlpSpec(**(spec_kwargs or {}))
        rng = np.random.default_rng(seed)
        n, sc, s = n_rays, n_coarse, self.s
        f32 = dict(device=self.dev, dtype=torch.float32)
        self.nets = {'coarse': NetState(self.spec, self.dev, rng), 'fine': NetState(self.spec, self.dev, rng)}
        self.run = [_Net('coarse', 'coarse', self.spec, self.nets['coarse'], n, sc, self.precision, self.dev, train),
                    _Net('fine', 'fine', self.spec, self.nets['fine'], n, s, self.precision, self.dev, train)]
        for name, kw in (aug or []):
            aspec = MlpSpec(**kw)
            for level, ss in (('coarse', sc), ('fine', s)):
                if level == 'fine' and not aug_fine:
                    continue
                tag = f'{name}_{level}'
                self.nets[tag] = NetState(aspec, self.dev, rng)
                self.run.append(_Net(tag, level, aspec, self.nets[tag], n, ss, self.precision, self.dev, train))
        # inputs (static buffers the host copies into)
        self.rays_o = torch.zeros(n, 3, **f32)
        self.rays_d = torch.zeros(n, 3, **f32)
        self.target_rgb = torch.zeros(n, 3, **f32)
        self.target_depth = torch.zeros(n, **f32)
        self.u_c = torch.zeros(n, sc, **f32)
        self.u_f = torch.zeros(n, n_fine, **f32)
        self.depth_mask = torch.zeros(n, dtype=torch.uint8, device=self.dev)
        self.depth_mask[:self.n_depth] = 1
        # intermediates shared by the nets of one level
        self.vdirs = torch.zeros(n, 3, **f32)
        self.rays_o_ndc = torch.zeros(n, 3, **f32)
        self.rays_d_ndc = torch.zeros(n, 3, **f32)
        self.focal = torch.full((n,), float(self.ndc['focal']) if self.ndc else 1.0, **f32)
        self.level = {lv: {'z': torch.zeros(n, ss, **f32), 'pts': torch.zeros(n * ss, 3, **f32)}
                      for lv, ss in (('coarse', sc), ('fine', s))}
        self.loss = torch.zeros(1, **f32)
        self._loss_structs = {}
        self.step_count = torch.zeros(1, dtype=torch.int32, device=self.dev)
        # augmented coarse nets run on their own streams, concurrently with the main
        # nets (they share only the read-only samples; their depth joins the main
        # stream for the consistency term)
        self.side = [_lib.new_stream(self.dev) for net in self.run[2:] if net.level == 'coarse'] \
            if concurrent_aug else []
        # the main coarse net's backward needs only its own forward: it runs on a
        # stream of its own while the fine net evaluates
        self.cb_stream = _lib.new_stream(self.dev) if (overlap_coarse and train) else None
        self.graph = None
        self.launches_per_step = None
        self.batcher = None

    def attach_batcher(self, batcher, seed=0):
        """Take every step's batch from ``batcher`` (a GpuRayBatcher over cached rays with
        cameras) inside the step itself: the batch gathers, the rays of its pixels
        (srf_pixel_rays, CommonUtils04.get_rays_tr), the stratified and inverse-CDF
        uniforms (srf_uniforms, keyed by the batch counter) and the counter's advance
        are enqueued with the render, so a captured step is the whole training
        iteration of Trainer10.train_one_iter.  No depth supervision in this form."""
        if batcher.num_rays != self.n or batcher.nsd:
            raise ValueError('the batcher must serve exactly the step\'s rays (no sparse-depth rows)')
        if 'intrinsics' not in batcher.out or 'extrinsics' not in batcher.out:
            raise ValueError('the batcher needs the cameras (intrinsics and extrinsics) to form rays')
        if self.ndc:
            raise NotImplementedError('batches from cached rays are supported for world-space rays')
        self.batcher = batcher
        self.batch_seed = int(seed) & ((1 << 64) - 1)
        self.n_depth = 0
        self.depth_mask.zero_()
        self._loss_structs = {}

    def _enqueue_batch(self, lib, st):
        b = self.batcher
        o = b.assemble()
        n = self.n
        _lib.check(lib.srf_pixel_rays(_vp(o['pixel_id']), _vp(o['intrinsics']), _vp(o['extrinsics']), n, 0,
                                      _vp(self.rays_o), _vp(self.rays_d), st), 'pixel_rays')
        self.target_rgb.copy_(o['target_rgb'])
        if self.perturb:
            for sid, u in enumerate((self.u_c, self.u_f)):
                _lib.check(lib.srf_uniforms(_vp(u), u.numel(), self.batch_seed, _vp(b.counter), sid, st), 'uniforms')

    @property
    def buf(self):
        """Per-net buffers keyed by net tag, with the level's depths under 'z'."""
        out = {}
        for net in self.run:
            d = dict(net.b)
            d['z'] = self.level[net.level]['z']
            out[net.name] = d
        return out

    # ------------------------------------------------------------ enqueue --
    def _composite_args(self, net, backward):
        b = net.b
        z = self.level[net.level]['z']
        a = _lib.CompositeArgs()
        a.n_rays, a.n_samples = self.n, z.shape[1]
        a.flags = (_lib.SRF_COMPOSITE_WHITE_BKGD if self.white else 0) | (_lib.SRF_COMPOSITE_NDC if self.ndc else 0)
        if self.precision != _lib.SRF_PRECISION_FP32 and a.n_samples <= 256:
            # the 16-bit steps take transmittance as exp of an exclusive prefix sum of
            # sigma delta; the FP32 plain step keeps the reference's cumprod form
            a.flags |= _lib.SRF_COMPOSITE_EXP_PREFIX
        a.distance_scale = 1.0
        a.sigma, a.rgb, a.z, a.rays_d = b['sigma'].data_ptr(), b['rgb'].data_ptr(), z.data_ptr(), \
            self.rays_d.data_ptr()
        if self.ndc:
            a.rays_o, a.rays_d_ndc = self.rays_o.data_ptr(), self.rays_d_ndc.data_ptr()
        if not backward:
            a.rgb_map, a.acc, a.depth = b['rgb_map'].data_ptr(), b['acc'].data_ptr(), b['depth'].data_ptr()
            a.depth_var, a.weights = b['depth_var'].data_ptr(), b['weights'].data_ptr()
            if self.ndc:
                a.depth_ndc, a.depth_var_ndc = b['depth_ndc'].data_ptr(), b['depth_var_ndc'].data_ptr()
        else:
            # the rgb / depth loss gradients come from the fused loss; g_depth carries
            # only the consistency term's share (main coarse net of the pair)
            if net is self.run[0] and self._consistency():
                a.g_depth = b['g_depth'].data_ptr()
            a.d_sigma, a.d_rgb = b['d_sigma'].data_ptr(), b['d_rgb'].data_ptr()
        return a

    def _consistency(self):
        """Whether an augmented coarse net's depth is a consistency target of the main coarse depth."""
        return self.consistency_weight > 0 and any(x.level == 'coarse' for x in self.run[2:])

    def _loss_args(self, net):
        """rgb MSE of this net (MSE14.compute_mse) plus, with depth-supervised rays, the
        L1 depth term, evaluated inside compositing (srf_composite_loss)."""
        key = net.name
        if key not in self._loss_structs:
            L = _lib.CompositeLoss()
            L.target_rgb, L.rgb_weight = self.target_rgb.data_ptr(), 1.0
            if self.n_depth > 0:
                L.target_depth, L.depth_mask = self.target_depth.data_ptr(), self.depth_mask.data_ptr()
                L.n_depth_rays, L.depth_weight, L.depth_squared = self.n_depth, float(self.depth_weight), 0
            L.loss = self.loss.data_ptr()
            self._loss_structs[key] = L
        return self._loss_structs[key]

    def _enqueue(self):
        lib = _lib.load()
        st = _P(torch.cuda.current_stream(self.dev).cuda_stream)
        chk = _lib.check
        n = self.n
        if self.batcher is not None:
            with F.nvtx_range('srf.batch'):
                self._enqueue_batch(lib, st)
        if self.ndc:
            h, w = self.ndc['h'], self.ndc['w']
            chk(lib.srf_ndc_rays(_vp(self.rays_o), _vp(self.rays_d), _vp(self.focal), _vp(self.focal), n, h, w,
                                 float(self.ndc['near']), _vp(self.rays_o_ndc), _vp(self.rays_d_ndc),
                                 _vp(self.vdirs), st), 'ndc_rays')
            po, pd = self.rays_o_ndc, self.rays_d_ndc
        else:
            chk(lib.srf_ndc_rays(None, _vp(self.rays_d), None, None, n, 1, 1, 0.0, None, None, _vp(self.vdirs),
                                 st), 'view_dirs')
            po, pd = self.rays_o, self.rays_d
        if self.train:
            self.loss.zero_()
        zc = self.level['coarse']['z']
        u_c, u_f = (self.u_c, self.u_f) if self.perturb else (None, None)
        chk(lib.srf_stratified_z(_vp(zc), _vp(u_c), n, self.sc, self.near, self.far, 0, st), 'stratified_z')
        main_coarse = self.run[0]
        main_stream = torch.cuda.current_stream(self.dev)
        side_of, done = {}, {}
        for level in ('coarse', 'fine'):
            torch.cuda.nvtx.range_push(f'srf.{level}')
            lv = self.level[level]
            ss = lv['z'].shape[1]
            if level == 'fine':
                chk(lib.srf_fine_z(_vp(lv['z']), _vp(zc), _vp(main_coarse.b['weights']), _vp(u_f), n, self.sc,
                                   self.sf, st), 'fine_z')
            chk(lib.srf_ray_points(_vp(po), _vp(pd), _vp(lv['z']), n, ss, _vp(lv['pts']), st), 'ray_points')
            if level == 'coarse' and self.side:
                fork = torch.cuda.Event()
                fork.record(main_stream)
                for net, side in zip((x for x in self.run[2:] if x.level == 'coarse'), self.side):
                    side.wait_event(fork)
                    side_of[net.name] = side
            for net in (x for x in self.run if x.level == level):
                b = net.b
                sp = _P(side_of[net.name].cuda_stream) if net.name in side_of else st
                chk(lib.srf_nerf_mlp_forward(ctypes.byref(net.spec.desc), net.state.pptr, _vp(lv['pts']),
                                             _vp(self.vdirs), ss, n * ss, None, _vp(b['sigma']), _vp(b['rgb']),
                                             self.precision, int(self.train), _vp(b['ws']), b['ws'].numel(),
                                             _vp(self.scaler), sp),
                    'mlp_forward')
                if self.train:
                    # the loss of this net's render is evaluated in the compositing
                    # epilogue; its gradient is recomputed inside the adjoint
                    chk(lib.srf_composite_forward_loss(ctypes.byref(self._composite_args(net, False)),
                                                       ctypes.byref(self._loss_args(net)), sp), 'composite_forward')
                else:
                    chk(lib.srf_composite_forward(ctypes.byref(self._composite_args(net, False)), sp),
                        'composite_forward')
                if net.name in side_of:
                    ev = torch.cuda.Event()
                    ev.record(side_of[net.name])
                    done[net.name] = ev   # its depth is final here
                    if self.train:
                        # an augmented net's gradients do not depend on the main nets:
                        # its backward follows right away on its own stream
                        self._backward(lib, net, sp)
            if level == 'coarse' and self.cb_stream is not None:
                cb = self.cb_stream
                ev = torch.cuda.Event()
                ev.record(main_stream)
                cb.wait_event(ev)
                self._coarse_backward(lib, main_coarse, done, cb)
            torch.cuda.nvtx.range_pop()
        if not self.train:
            for ev in done.values():
                main_stream.wait_event(ev)
            return
        torch.cuda.nvtx.range_push('srf.backward')
        if self.cb_stream is None:
            self._coarse_backward(lib, main_coarse, done, main_stream)
        for net in reversed(self.run):
            if net.name not in side_of and net is not main_coarse:
                self._backward(lib, net, st)
        for side in list(side_of.values()) + ([self.cb_stream] if self.cb_stream is not None else []):
            main_stream.wait_stream(side)
        torch.cuda.nvtx.range_pop()
        torch.cuda.nvtx.range_push('srf.adam')
        chk(lib.srf_counter_add(_vp(self.step_count), 1, self.found_inf, st), 'counter')
        for net in self.nets.values():
            chk(lib.srf_adam_step(_vp(net.flat), _vp(net.grad), _vp(net.m), _vp(net.v), net.flat.numel(), self.lr,
                                  self.betas[0], self.betas[1], self.eps, 0.0, 1, _vp(self.step_count),
                                  self.found_inf, st), 'adam')
        if self.scaler is not None:
            chk(lib.srf_loss_scaler_update(_vp(self.scaler), 2.0, 0.5, 2000, st), 'loss_scaler_update')
        if self.batcher is not None:
            self.batcher.advance()
        torch.cuda.nvtx.range_pop()

    def _coarse_backward(self, lib, main_coarse, done, stream):
        """The consistency term (augmented coarse depth as a detached target of the
        main coarse depth) and the main coarse net's backward, on ``stream``."""
        sp = _P(stream.cuda_stream)
        if self._consistency():
            # the consistency terms accumulate into the main coarse depth gradient
            with torch.cuda.stream(stream):
                main_coarse.b['g_depth'].zero_()
        for net in self.run[2:]:
            if net.level == 'coarse' and self.consistency_weight > 0:
                if net.name in done:
                    stream.wait_event(done[net.name])
                _lib.check(lib.srf_depth_mse_loss(_vp(main_coarse.b['depth']), _vp(net.b['depth']), None, self.n,
                                                  self.consistency_weight, 0, _vp(self.loss),
                                                  _vp(main_coarse.b['g_depth']), None, sp), 'consistency')
        self._backward(lib, main_coarse, sp)

    def _backward(self, lib, net, stream):
        b = net.b
        ss = self.level[net.level]['z'].shape[1]
        _lib.check(lib.srf_composite_backward_loss(ctypes.byref(self._composite_args(net, True)),
                                                   ctypes.byref(self._loss_args(net)), stream), 'composite_backward')
        _lib.check(lib.srf_nerf_mlp_backward(ctypes.byref(net.spec.desc), net.state.pptr, _vp(b['d_sigma']),
                                             _vp(b['d_rgb']), ss, self.n * ss, net.state.gptr, 0, self.precision,
                                             _vp(b['ws']), b['ws'].numel(), _vp(self.scaler), stream),
                   'mlp_backward')

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
        out = {}
        for net in self.run:
            for k in ('rgb_map', 'acc', 'depth', 'depth_var', 'weights', 'sigma') + (('depth_ndc',) if self.ndc else ()):
                out[f'{k}_{net.name}'] = net.b[k]
            out[f'z_{net.name}'] = self.level[net.level]['z']
        return out


def main(argv=None):
    """Run a fused training step on synthetic data and print ms/step:

        python -m simple_rf_gb300.train_step --rays 4096 --steps 10 --warmup 3 [--precision fp32] [--eager]
            [--config nerf|nerf_pair] [--mlp-path default|fused|layers]
    """
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument('--rays', type=int, default=4096)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--precision', default='bf16', choices=['bf16', 'fp16', 'fp32'])
    ap.add_argument('--eager', action='store_true', help='launch kernels directly instead of replaying a CUDA graph')
    ap.add_argument('--config', default='nerf', choices=['nerf', 'nerf_pair'])
    ap.add_argument('--mlp-path', default='default', choices=['default', 'fused', 'layers'],
                    help='16-bit MLP forward: the library default (fused for forward-only calls), the fused '
                         'kernel for every forward, or one kernel per layer')
    args = ap.parse_args(argv)
    from . import build as _build
    _build.build()
    if args.mlp_path != 'default':
        _lib.load().srf_nerf_mlp_fused_path(2 if args.mlp_path == 'fused' else 0)
    dev = torch.device('cuda')
    step, batch_fn = make_step(args.config, args.rays, args.precision, dev)
    step.set_batch(*batch_fn(1, dev))
    if not args.eager:
        step.capture(warmup=1)
    for _ in range(args.warmup):
        step.step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    # the timed steps are the range a profiler started with profiling off captures
    torch.cuda.profiler.start()
    with F.nvtx_range('srf.timed_steps'):
        for _ in range(args.steps):
            step.step()
    e1.record()
    torch.cuda.profiler.stop()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / max(args.steps, 1)
    print(json.dumps({'config': args.config, 'rays': args.rays, 'precision': args.precision, 'graph': not args.eager,
                      'ms_per_step': round(ms, 4), 'rays_per_s': round(args.rays / ms * 1e3, 1),
                      'loss': float(step.loss.item())}))


def synthetic_batch(n_rays, n_coarse, n_fine, seed, device='cpu', pin=False):
    """Synthetic inputs of the 4096-ray training step: o ~ N(0, 0.1^2), d = normalize(N(0, I)), rgb
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


def synthetic_batch_ndc(n_rays, n_coarse, n_fine, seed, device='cpu', pin=False):
    """Forward-facing synthetic inputs: origins on the z = -1 plane with x, y ~ U[-1, 1];
    directions normalise (U[-0.2, 0.2], U[-0.2, 0.2], U[-1.2, -0.8]); rgb targets
    ~ U[0,1]^3; depth targets unused (zeros); stratified/pdf uniforms ~ U[0,1)."""
    g = torch.Generator().manual_seed(seed)
    o = torch.rand(n_rays, 3, generator=g) * 2 - 1
    o[:, 2] = -1.0
    d = torch.rand(n_rays, 3, generator=g)
    d[:, :2] = d[:, :2] * 0.4 - 0.2
    d[:, 2] = -(d[:, 2] * 0.4 + 0.8)
    d = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    t_rgb = torch.rand(n_rays, 3, generator=g)
    t_depth = torch.zeros(n_rays)
    u_c = torch.rand(n_rays, n_coarse, generator=g)
    u_f = torch.rand(n_rays, n_fine, generator=g)
    out = [o, d, t_rgb, t_depth, u_c, u_f]
    if pin:
        out = [x.pin_memory() for x in out]
    if str(device) != 'cpu':
        out = [x.to(device) for x in out]
    return out


AUG_VIEWS = ('views_augmentation', dict(points_pe_degree=4, use_view_dirs=False, view_dependent_rgb=False))
NDC_LLFF = dict(h=378, w=504, focal=400.0, near=1.0)


def make_step(config, n_rays=4096, precision='bf16', device='cuda', seed=0, **kw):
    """The two training-step workloads by name:

    'nerf'      -- world rays, coarse + fine nets, white background, 25% depth-supervised rays;
    'nerf_pair' -- NDC forward-facing rays (H 378, W 504, focal 400, near 1), main coarse + fine
                   nets plus a coarse augmented net (PE L=4 on xyz, no view directions) on the
                   same coarse samples, its depth a 0.1-weighted squared-error target of the
                   main coarse depth, no sparse-depth rays, black background.
    Returns (step, batch_fn) where batch_fn(seed, device, pin) makes matching inputs.
    """
    if config == 'nerf':
        step = NerfTrainStep(n_rays, 64, 128, precision=precision, device=device, seed=seed, **kw)
        return step, lambda sd, dev, pin=False: synthetic_batch(n_rays, 64, 128, sd, dev, pin)
    if config == 'nerf_pair':
        args = dict(white_bkgd=False, depth_fraction=0.0, ndc=NDC_LLFF, aug=[AUG_VIEWS], consistency_weight=0.1)
        args.update(kw)
        step = NerfTrainStep(n_rays, 64, 128, precision=precision, device=device, seed=seed, **args)
        return step, lambda sd, dev, pin=False: synthetic_batch_ndc(n_rays, 64, 128, sd, dev, pin)
    raise ValueError(f'unknown training-step workload {config!r}')


if __name__ == '__main__':
    main()
