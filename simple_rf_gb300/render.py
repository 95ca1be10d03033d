"""Full-image rendering of the Simple-NeRF main + augmented pair in ray chunks.

The test-time render path of ``SimpleNeRF.forward`` (src/models/SimpleNeRF17.py:104-157:
``batchify_rays`` splits the rays into ``chunk``-sized pieces and ``render_rays``
runs each, :133-157) on the srf_gb300 kernels: per chunk, NDC warp, stratified
samples without jitter, coarse networks, compositing, deterministic inverse-CDF
fine samples, fine network, compositing.  The reference runs augmented nets only
in training (:244); here they are rendered explicitly alongside the main nets so
the pair's whole forward is measured.  A chunk is one CUDA graph replay; the
last, partial chunk replays the same graph on a padded batch and keeps only its
real rays.

    python -m simple_rf_gb300.render --views 8 --height 378 --width 504 --chunk 65536
"""
import argparse
import json

import torch

from . import _lib
from . import functional as F
from .train_step import make_step


class NerfPairRenderer:
    """Chunked forward render of the main coarse + fine nets and the augmented coarse net."""

    def __init__(self, chunk=65536, precision='bf16', device='cuda', seed=0, graph=True, nets=None):
        self.chunk = int(chunk)
        self.step, _ = make_step('nerf_pair', self.chunk, precision, device, seed=seed, train=False, perturb=False)
        if nets is not None:
            for tag, state in nets.items():
                self.step.nets[tag].flat.copy_(state.flat)
        self.graph = bool(graph)
        self._captured = False

    @property
    def nets(self):
        return self.step.nets

    def render(self, rays_o, rays_d, keep=('rgb', 'depth', 'acc')):
        """World rays (N, 3) -> {net: {'rgb': (N, 3), 'depth': (N,), 'acc': (N,)}}; ``keep`` may
        also name 'z' (the net's sample depths) and 'weights'."""
        n = rays_o.shape[0]
        dev = rays_o.device
        st = self.step

        def src(net, k):
            if k == 'z':
                return st.level[net.level]['z']
            return net.b['rgb_map' if k == 'rgb' else k]

        out = {net.name: {k: torch.empty((n,) + tuple(src(net, k).shape[1:]), device=dev) for k in keep}
               for net in st.run}
        for i in range(0, n, self.chunk):
            k = min(self.chunk, n - i)
            st.rays_o[:k].copy_(rays_o[i:i + k])
            st.rays_d[:k].copy_(rays_d[i:i + k])
            if self.graph and not self._captured:
                # one eager pass on real rays, then the capture (which does not execute)
                st.capture(warmup=1)
                self._captured = True
            st.step()
            for net in st.run:
                for key, dst in out[net.name].items():
                    dst[i:i + k].copy_(src(net, key)[:k])
        return out

    def samples_per_ray(self):
        return sum(self.step.level[net.level]['z'].shape[1] for net in self.step.run)


def synthetic_views(n_views, height, width, focal=400.0, seed=0, device='cuda'):
    """Forward-facing cameras: identity rotation, translations ~ U[-0.1, 0.1]^3,
    principal point at the image centre.  Returns (pixel_id (N,3) int32 = (view, x, y),
    intrinsics (V,3,3), extrinsics (V,4,4) camera-to-world)."""
    g = torch.Generator().manual_seed(seed)
    k = torch.tensor([[focal, 0.0, width / 2.0], [0.0, focal, height / 2.0], [0.0, 0.0, 1.0]])
    intr = k.expand(n_views, 3, 3).contiguous()
    ext = torch.eye(4).expand(n_views, 4, 4).contiguous()
    ext[:, :3, 3] = torch.rand(n_views, 3, generator=g) * 0.2 - 0.1
    v, y, x = torch.meshgrid(torch.arange(n_views), torch.arange(height), torch.arange(width), indexing='ij')
    pid = torch.stack([v, x, y], -1).reshape(-1, 3).to(torch.int32)
    return pid.to(device), intr.to(device), ext.to(device)


def pixel_rays(pid, intr, ext):
    """World rays of every pixel id (per-ray camera matrices gathered by view)."""
    view = pid[:, 0].long()
    return F.pixel_rays(pid, intr[view].contiguous(), ext[view].contiguous())


def _time_render(r, o, d, reps, profile=False):
    """ms per full render after a capture + warm-up chunk; with profile the timed
    renders are the range a profiler started with profiling off captures."""
    r.render(o[:r.chunk], d[:r.chunk])            # capture + warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if profile:
        torch.cuda.profiler.start()
    e0.record()
    for _ in range(reps):
        out = r.render(o, d)
    e1.record()
    e1.synchronize()
    if profile:
        torch.cuda.profiler.stop()
    return e0.elapsed_time(e1) / reps, out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('--views', type=int, default=8)
    ap.add_argument('--height', type=int, default=378)
    ap.add_argument('--width', type=int, default=504)
    ap.add_argument('--chunk', type=int, default=65536)
    ap.add_argument('--reps', type=int, default=2)
    ap.add_argument('--fp32-rays', type=int, default=4 * 65536,
                    help='rays of the image rendered by the FP32 plain path (a prefix of the full set)')
    ap.add_argument('--mlp-path', default='default', choices=['default', 'fused', 'layers'],
                    help='16-bit MLP forward: the library default (fused for forward-only calls), the fused '
                         'kernel for every forward, or one kernel per layer')
    args = ap.parse_args(argv)
    from . import build as _build
    _build.build()
    if args.mlp_path != 'default':
        _lib.load().srf_nerf_mlp_fused_path(2 if args.mlp_path == 'fused' else 0)
    dev = torch.device('cuda')
    pid, intr, ext = synthetic_views(args.views, args.height, args.width, device=dev)
    o, d = pixel_rays(pid, intr, ext)
    n = o.shape[0]
    lib = _lib.load()
    res = {'workload': f'nerf_pair_full_image_render_{args.views}x{args.width}x{args.height}',
           'rays': n, 'chunk': args.chunk}
    r = NerfPairRenderer(args.chunk, 'bf16', dev)
    l0 = lib.srf_launch_count()
    ms, out = _time_render(r, o, d, args.reps, profile=True)
    spr = r.samples_per_ray()
    res['bf16'] = {'ms': round(ms, 3), 'rays_per_s': round(n / ms * 1e3, 1),
                   'samples_per_s': round(n * spr / ms * 1e3, 1), 'samples_per_ray': spr,
                   'gpu_launches_per_chunk': r.step.launches_per_step,
                   'mean_rgb_fine': float(out['fine']['rgb'].mean().item())}
    del r, out
    torch.cuda.empty_cache()
    nf = min(args.fp32_rays, n)
    r32 = NerfPairRenderer(args.chunk, 'fp32', dev, graph=False)
    ms32, _ = _time_render(r32, o[:nf], d[:nf], 1)
    res['fp32_plain'] = {'rays': nf, 'ms': round(ms32, 3), 'rays_per_s': round(nf / ms32 * 1e3, 1)}
    res['speedup_bf16_vs_fp32_plain'] = round(res['bf16']['rays_per_s'] / res['fp32_plain']['rays_per_s'], 2)
    res['gpu_launches_total'] = int(lib.srf_launch_count() - l0)
    print(json.dumps(res))


if __name__ == '__main__':
    main()
