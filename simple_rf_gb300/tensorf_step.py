"""TensoRF training steps over the drop-in VM modules (SimpleTensoRF.render_rays ->
LowRankTensor.forward, src/models/SimpleTensoRF09.py:194-351, 701-761; the
reference's Trainer10.train_one_iter, src/Trainer10.py:65-115, around them):
forward of every model on its ray batch, rgb MSE, backward, and one
multi-tensor Adam launch over every parameter group.

TensorfTrainStep runs uncaptured (two host reads of sample counts per step);
TensorfGraphStep captures the whole step as one CUDA graph.
"""
import collections
import ctypes

import torch

from . import _lib
from . import functional as F
from .tensorf_model import _side_stream, forward_models


class TensorfTrainStep:
    """forward (every model) -> rgb MSE -> backward -> Adam (one srf_adam_multi_step launch).
    Samples march from ``near`` to ``far`` along each ray inside each model's box
    (SimpleTensoRF09.py:388-400)."""

    def __init__(self, models, lr_tensor=0.02, lr_network=1e-3, near=2.0, far=6.0):
        self.models = models
        self.near, self.far = float(near), float(far)
        self.params = []
        for tm in models:
            tensor_ps = list(tm.matrices_density) + list(tm.vectors_density) + list(tm.matrices_color) + \
                list(tm.vectors_color)
            net_ps = [tm.basis_matrix_color.weight] + list(tm.color_predictor.parameters())
            self.params += [(p, lr_tensor) for p in tensor_ps] + [(p, lr_network) for p in net_ps]
        self.state = [(torch.zeros_like(p), torch.zeros_like(p)) for p, _ in self.params]
        self.t = 0
        self.last = {}

    def step(self, o, d, t_rgb, u):
        vd = F.view_dirs(d)
        loss = 0.0
        calls = []
        for i, tm in enumerate(self.models):
            bbox, s, step = tm.host_geometry()
            z = F.aabb_z(o, d, s, bbox, self.near, self.far, step, u[:, i].contiguous())
            calls.append((tm, {'z_vals': z, 'rays_o': o, 'rays_d': d, 'view_dirs': vd}))
        # both models' phases side by side: two host reads of sample counts per step
        with F.nvtx_range('srf.tensorf.forward'):
            for out in forward_models(calls, retraw=False):
                loss = loss + torch.mean(torch.mean((out['rgb'] - t_rgb) ** 2, -1))
        counts = [dict(tm.last_sample_counts) for tm in self.models]
        for p, _ in self.params:
            p.grad = None
        with F.nvtx_range('srf.tensorf.backward'):
            loss.backward()
        self.t += 1
        with F.nvtx_range('srf.tensorf.adam'):
            F.adam_multi_step([(p.data, p.grad.contiguous(memory_format=_fmt(p)), m, v, lr)
                               for (p, lr), (m, v) in zip(self.params, self.state) if p.grad is not None],
                              step=self.t, beta1=0.9, beta2=0.99, eps=1e-8)
        self.last = {'loss': loss.detach(), 'samples': counts}
        return loss


class TensorfGraphStep:
    """The TensorfTrainStep step (both models' forward, rgb MSE, backward, one
    multi-tensor Adam launch) captured as one CUDA graph for a fixed ray count.

    A replay cannot read the compacted sample counts on the host, so the
    captured step sizes the valid- and surface-sample launches by capacities:
    15% above the counts of an uncaptured counting pass, rounded up to 1024
    rows.  Rows past a device count are zero points whose outputs nothing reads
    and whose gradients are zero, so a replay computes what TensorfTrainStep
    computes (up to the grouping of the sums over samples).  A count above its
    capacity raises a device flag that skips the Adam update and the step
    counter; the call reads the flag once its replay has ended and, when it is
    set, re-captures with capacities 25% above the counts and redoes the batch.
    Padding rows still cost the renderer MLP and basis passes their full work,
    so when the largest counts of the last 8 replays fall below 1 / 1.4 of the
    capacities (the surface count drops as the density field trains) the next
    call re-captures with capacities 15% above those counts.
    """

    MARGIN = 1.15     # capacities above the counts at a capture
    REGROW = 1.25     # ... at a re-capture after an overflow
    SHRINK = 1.4      # capacities this far above the counts are re-captured at SHRINK_TO
    SHRINK_TO = 1.15
    WINDOW = 8        # replays whose largest counts a shrink keeps room for
    ROUND = 1024

    def __init__(self, models, n_rays, lr_tensor=0.02, lr_network=1e-3, state=None, step_dev=None, near=2.0,
                 far=6.0):
        self.models = models
        self.near, self.far = float(near), float(far)
        self.n = int(n_rays)
        dev = models[0].matrices_density[0].device
        self.dev = dev
        self.params = []
        for tm in models:
            tensor_ps = list(tm.matrices_density) + list(tm.vectors_density) + list(tm.matrices_color) + \
                list(tm.vectors_color)
            net_ps = [tm.basis_matrix_color.weight] + list(tm.color_predictor.parameters())
            self.params += [(p, lr_tensor) for p in tensor_ps] + [(p, lr_network) for p in net_ps]
        self.state = state if state is not None else [(torch.zeros_like(p), torch.zeros_like(p))
                                                      for p, _ in self.params]
        i32 = dict(dtype=torch.int32, device=dev)
        self.step_dev = step_dev if step_dev is not None else torch.zeros(1, **i32)
        self.ovf = torch.zeros(1, **i32)
        k = len(models)
        self.caps_dev = torch.zeros(2 * k, **i32)
        self.flags_dev = torch.zeros(1 + 2 * k, **i32)
        self.flags_host = torch.zeros(1 + 2 * k, dtype=torch.int32, pin_memory=True)
        self.loss = torch.zeros(1, device=dev)
        f32 = dict(device=dev, dtype=torch.float32)
        self.o, self.d = torch.zeros(self.n, 3, **f32), torch.zeros(self.n, 3, **f32)
        self.t_rgb, self.u = torch.zeros(self.n, 3, **f32), torch.zeros(self.n, k, **f32)
        self.caps = None
        self.graph = None
        self.done = torch.cuda.Event()
        self.launches_per_step = None
        self.recaptures = 0
        self.shrinks = 0
        self._recent = collections.deque(maxlen=self.WINDOW)   # counts of the last replays
        self._shrink_to = None

    def _calls(self):
        vd = F.view_dirs(self.d)
        calls = []
        for i, tm in enumerate(self.models):
            bbox, s, step = tm.host_geometry()
            z = F.aabb_z(self.o, self.d, s, bbox, self.near, self.far, step, self.u[:, i].contiguous())
            calls.append((tm, {'z_vals': z, 'rays_o': self.o, 'rays_d': self.d, 'view_dirs': vd}))
        return calls

    def _body(self, dry):
        self.ovf.zero_()
        calls = self._calls()
        # every model after the first on a stream of its own (forked from and joined
        # back to the capturing stream), as forward_models runs them uncaptured; the
        # backward of each model's kernels follows its forward's stream
        main = torch.cuda.current_stream(self.dev)
        streams = [main] + [_side_stream(self.dev, i) for i in range(1, len(calls))]
        losses, states = [], []
        for (tm, inp), sm, (cv, cs) in zip(calls, streams, self.caps):
            sm.wait_stream(main)
            with torch.cuda.stream(sm):
                st = tm.forward_begin(inp)
                tm.forward_density(st, cv, capacity=True)
                out = tm.forward_color(st, cs, retraw=False, capacity=True)
                losses.append(torch.mean(torch.mean((out['rgb'] - self.t_rgb) ** 2, -1)))
                states.append(st)
        for sm in streams[1:]:
            main.wait_stream(sm)
        loss = losses[0]
        for x in losses[1:]:
            loss = loss + x
        counts = torch.cat([torch.cat([st['cnt_v'].reshape(1), st['cnt_s'].reshape(1)]) for st in states])
        self.ovf.copy_((counts > self.caps_dev).any().to(torch.int32).reshape(1))
        if dry:
            self.ovf.fill_(1)   # the dry run before a capture leaves parameters and step count alone
        for p, _ in self.params:
            p.grad = None
        loss.backward()
        st = ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        _lib.call('srf_counter_add', F._ptr(self.step_dev), 1, F._ptr(self.ovf), st)
        F.adam_multi_step([(p.data, p.grad.contiguous(memory_format=_fmt(p)), m, v, lr)
                           for (p, lr), (m, v) in zip(self.params, self.state) if p.grad is not None],
                          step=1, beta1=0.9, beta2=0.99, eps=1e-8, step_dev=self.step_dev, skip_dev=self.ovf)
        self.loss.copy_(loss.detach().reshape(1))
        self.flags_dev[:1].copy_(self.ovf)
        self.flags_dev[1:].copy_(counts)
        self.flags_host.copy_(self.flags_dev, non_blocking=True)

    def _counts(self):
        with torch.no_grad():
            forward_models(self._calls(), retraw=False)
        return [(tm.last_sample_counts['valid'], tm.last_sample_counts['surface']) for tm in self.models]

    @classmethod
    def capacities(cls, counts, margin):
        """(valid, surface) launch capacities for per-model (valid, surface)
        sample counts: margin above each count, rounded up to the next multiple of
        ROUND rows (always above the count, so a capacity of 0 never occurs)."""
        def cap(x):
            return (int(x * margin) // cls.ROUND + 1) * cls.ROUND
        return [(cap(v), cap(s)) for v, s in counts]

    def _capture(self, counts, margin):
        self.caps = self.capacities(counts, margin)
        self.caps_dev.copy_(torch.tensor([c for pair in self.caps for c in pair], dtype=torch.int32))
        self.graph = None
        torch.cuda.synchronize(self.dev)
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(side):
            self._body(dry=True)
        torch.cuda.current_stream(self.dev).wait_stream(side)
        torch.cuda.synchronize(self.dev)
        lib = _lib.load()
        l0 = lib.srf_launch_count()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._body(dry=False)
        self.launches_per_step = int(lib.srf_launch_count() - l0)
        self.graph = g

    def _replay(self, batch):
        for dst, src in zip((self.o, self.d, self.t_rgb, self.u), batch):
            dst.copy_(src)
        self.graph.replay()
        self.done.record()

    def step(self, o, d, t_rgb, u):
        """One training step on this batch (device tensors); returns the loss
        buffer.  The host waits for the replay to read its overflow flag: a replay
        that overflowed a capacity (its update skipped) is re-captured with
        larger capacities and redone before the call returns."""
        batch = (o, d, t_rgb, u)
        if self.graph is None:
            for dst, src in zip((self.o, self.d, self.t_rgb, self.u), batch):
                dst.copy_(src)
            self._capture(self._counts(), self.MARGIN)
        elif self._shrink_to is not None:
            for dst, src in zip((self.o, self.d, self.t_rgb, self.u), batch):
                dst.copy_(src)
            self.shrinks += 1
            self._capture(self._shrink_to, self.SHRINK_TO)
            self._shrink_to = None
            self._recent.clear()
        self._replay(batch)
        self.done.synchronize()
        while int(self.flags_host[0]):
            # the replay's counts are the full counts even where they overflowed
            self.recaptures += 1
            peak = self._host_counts()
            for c in self._recent:
                peak = [(max(a[0], b[0]), max(a[1], b[1])) for a, b in zip(peak, c)]
            self._capture(peak, max(self.MARGIN, self.REGROW))
            self._replay(batch)
            self.done.synchronize()
        # capacities far above the counts of every recent batch (the surface count
        # falls as the density field trains) cost each replay the padded rows' full
        # work: the next call re-captures them at SHRINK_TO above the recent maxima
        self._recent.append(self._host_counts())
        if len(self._recent) == self._recent.maxlen:
            peak = [tuple(max(c[i][k] for c in self._recent) for k in range(2)) for i in range(len(self.models))]
            if any(cap > self.SHRINK * max(cnt, self.ROUND) for caps, cnts in zip(self.caps, peak)
                   for cap, cnt in zip(caps, cnts)):
                self._shrink_to = peak
        return self.loss

    def _host_counts(self):
        c = self.flags_host[1:].tolist()
        return [(c[2 * i], c[2 * i + 1]) for i in range(len(self.models))]

    def sample_counts(self):
        """Valid and surface sample counts of the last finished replay, per model."""
        self.done.synchronize()
        c = self.flags_host[1:].tolist()
        return [{'marched': None, 'valid': c[2 * i], 'surface': c[2 * i + 1]} for i in range(len(self.models))]


def _fmt(p):
    return torch.channels_last if p.dim() == 4 and p.is_contiguous(memory_format=torch.channels_last) else \
        torch.contiguous_format
