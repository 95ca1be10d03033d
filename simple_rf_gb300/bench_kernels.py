"""Kernel-level benchmarks of the hot-path kernels, one launch shape at a time.

    python -m simple_rf_gb300.bench_kernels gemm --m 786432 --k 256 --n 256
    python -m simple_rf_gb300.bench_kernels wgrad --m 786432 --n 256 --k 256
    python -m simple_rf_gb300.bench_kernels composite --rays 4096 --samples 192 [--backward]
    python -m simple_rf_gb300.bench_kernels vm --rays 1216 --samples 1024 --comps 48 [--kind density] [--backward]
    python -m simple_rf_gb300.bench_kernels mlp --m 786432 [--mlp-path fused|layers] [--store] [--precision fp16]

Each prints one JSON line: the average launch time over --reps launches
(CUDA events on the launching stream, after --warmup launches) and the achieved
FLOP/s and algorithmic bytes/s.  With --reps 1 --warmup 0 it launches the kernel
exactly once (for profilers).
"""
import argparse
import ctypes
import json

import torch

from . import _lib

_P = ctypes.c_void_p


def _p(t):
    return None if t is None else _P(t.data_ptr())


def _st():
    return _P(torch.cuda.current_stream().cuda_stream)


def _time(fn, reps, warmup):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3 / max(reps, 1)


def gemm(args):
    m, k, n = args.m, args.k, args.n
    g = torch.Generator(device='cuda').manual_seed(0)
    x = torch.randn(m, k, device='cuda', generator=g).to(torch.bfloat16)
    w = (torch.randn(n, k, device='cuda', generator=g) * 0.05).to(torch.bfloat16)
    b = torch.zeros(n, device='cuda')
    y = torch.empty(m, n, device='cuda', dtype=torch.bfloat16)
    # --dgrad: the backward-data form (ReLU mask of a forward activation, column sums, no bias)
    mask = torch.randn(m, n, device='cuda', generator=g).to(torch.bfloat16) if args.dgrad else None
    colsum = torch.zeros(n, device='cuda') if args.dgrad else None

    def run():
        _lib.call('srf_bf16_linear', _p(y), n, _p(x), k, k, None, 0, 0, _p(w), k, n, 0, None if args.dgrad else _p(b),
                  m, n, 0 if args.dgrad else 1, _p(mask), n if args.dgrad else 0, _p(colsum), _st())
    t = _time(run, args.reps, args.warmup)
    flops = 2.0 * m * n * k
    nbytes = (m * k + m * n * (2 if args.dgrad else 1) + n * k) * 2
    return {'kernel': 'tc_gemm_kernel', 'form': 'dgrad (mask + colsum)' if args.dgrad else 'forward (bias + ReLU)',
            'm': m, 'k': k, 'n': n, 'ms': t * 1e3, 'tflops': flops / t / 1e12, 'gbs': nbytes / t / 1e9,
            'bytes': nbytes}


def wgrad(args):
    m, k, n = args.m, args.k, args.n
    lib = _lib.load()
    g = torch.Generator(device='cuda').manual_seed(0)
    dz = torch.randn(m, n, device='cuda', generator=g).to(torch.bfloat16)
    x = torch.randn(m, k, device='cuda', generator=g).to(torch.bfloat16)
    nb = lib.srf_bf16_wgrad_workspace_size(n, k)
    part = torch.empty(nb // 4, device='cuda')
    sp = ctypes.c_int()

    def run():
        _lib.call('srf_bf16_wgrad', _p(part), nb, ctypes.byref(sp), _p(dz), n, n, _p(x), k, k, None, 0, 0, m, _st())
    t = _time(run, args.reps, args.warmup)
    flops = 2.0 * m * n * k
    nbytes = (m * n + m * k) * 2 + sp.value * n * k * 4
    return {'kernel': 'tc_wgrad_kernel', 'm': m, 'k': k, 'n': n, 'splits': sp.value, 'ms': t * 1e3,
            'tflops': flops / t / 1e12, 'gbs': nbytes / t / 1e9, 'bytes': nbytes}


def composite(args):
    """Compositing forward (or, with --backward, the reverse-scan adjoint, which
    recomputes the forward scan) over rays x samples."""
    nr, s = args.rays, args.samples
    g = torch.Generator(device='cuda').manual_seed(0)
    sigma = torch.rand(nr, s, device='cuda', generator=g)
    rgb = torch.rand(nr, s, 3, device='cuda', generator=g)
    z = torch.sort(torch.rand(nr, s, device='cuda', generator=g) * 4 + 2, 1)[0]
    d = torch.randn(nr, 3, device='cuda', generator=g)
    outs = {k: torch.empty(nr, 3 if k == 'rgb_map' else 1, device='cuda') for k in ('rgb_map', 'acc', 'depth', 'dv')}
    w = torch.empty(nr, s, device='cuda')
    a = _lib.CompositeArgs()
    a.n_rays, a.n_samples, a.flags, a.distance_scale = nr, s, _lib.SRF_COMPOSITE_WHITE_BKGD, 1.0
    a.sigma, a.rgb, a.z, a.rays_d = sigma.data_ptr(), rgb.data_ptr(), z.data_ptr(), d.data_ptr()
    if args.backward:
        g_rgb = torch.randn(nr, 3, device='cuda', generator=g)
        g_depth = torch.randn(nr, device='cuda', generator=g)
        d_sigma = torch.empty(nr, s, device='cuda')
        d_rgb = torch.empty(nr, s, 3, device='cuda')
        a.g_rgb, a.g_depth, a.d_sigma, a.d_rgb = g_rgb.data_ptr(), g_depth.data_ptr(), d_sigma.data_ptr(), \
            d_rgb.data_ptr()
        name = 'srf_composite_backward'
        # reads sigma, rgb, z; writes d_sigma, d_rgb
        nbytes = nr * s * (4 + 12 + 4 + 4 + 12) + nr * (12 + 12 + 4)
    else:
        a.rgb_map, a.acc, a.depth, a.depth_var, a.weights = (outs['rgb_map'].data_ptr(), outs['acc'].data_ptr(),
                                                             outs['depth'].data_ptr(), outs['dv'].data_ptr(),
                                                             w.data_ptr())
        name = 'srf_composite_forward'
        # reads sigma, rgb, z; writes weights
        nbytes = nr * s * (4 + 12 + 4 + 4) + nr * (12 + 12)

    def run():
        _lib.call(name, ctypes.byref(a), _st())
    t = _time(run, args.reps, args.warmup)
    return {'kernel': 'composite_bwd_kernel' if args.backward else 'composite_fwd_kernel', 'rays': nr, 'samples': s,
            'ms': t * 1e3, 'gbs': nbytes / t / 1e9, 'bytes': nbytes}


def vm_points(n_rays, samples, seed=0):
    """Normalised sample points in ray order (what the renderer hands the VM
    lookups): rays through the box, ``samples`` evenly spaced points on each."""
    g = torch.Generator(device='cuda').manual_seed(seed)
    o = torch.rand(n_rays, 3, device='cuda', generator=g) * 2 - 1
    e = torch.rand(n_rays, 3, device='cuda', generator=g) * 2 - 1
    t = torch.linspace(0, 1, samples, device='cuda')
    return (o[:, None, :] + (e - o)[:, None, :] * t[None, :, None]).reshape(-1, 3).contiguous()


def vm(args):
    """VM plane/line gathers (or, with --backward, the 128-bit scatter-add
    adjoint) at a res^3 grid with R components per plane/line.  Algorithmic
    bytes per point: 3 planes x 4 corners + 3 lines x 2 ends, R floats each
    (3456 B at R = 48, 1152 B at R = 16), plus the point and the features; the
    backward reads d_features and both factors' corners and read-modify-writes
    the gradient corners (3x the corner bytes).  The
    grid itself (3 x res^2 x R x 4 B, 51.8 MB at 300^2 x 48) stays in the 129 MB
    L2, so the fraction of the HBM copy peak can exceed 1."""
    from .tensorf import VmGridTensors, _grid_struct
    res, r, p = args.res, args.comps, args.rays * args.samples
    g = torch.Generator(device='cuda').manual_seed(0)
    planes = [(torch.randn(1, r, res, res, device='cuda', generator=g) * 0.1).contiguous(
        memory_format=torch.channels_last) for _ in range(3)]
    lines = [(torch.randn(1, r, res, 1, device='cuda', generator=g) * 0.1).contiguous(
        memory_format=torch.channels_last) for _ in range(3)]
    grid = VmGridTensors(planes, lines, [res] * 3)
    gs = _grid_struct(grid.res, grid.planes, grid.lines)
    pts = vm_points(args.rays, args.samples)
    color = args.kind == 'color'
    feat = torch.empty(p, 3 * r if color else 1, device='cuda')
    corner = (3 * 4 + 3 * 2) * r * 4
    if args.backward:
        gp = [torch.zeros_like(x) for x in planes]
        gl = [torch.zeros_like(x) for x in lines]
        gg = _grid_struct(grid.res, gp, gl)
        dfeat = torch.randn(p, feat.shape[1], device='cuda', generator=g)
        name = 'srf_vm_color_backward' if color else 'srf_vm_density_backward'

        def run():
            _lib.call(name, ctypes.byref(gg), ctypes.byref(gs), _p(pts), p, _p(dfeat), _st())
        nbytes = p * (3 * corner + 12 + feat.shape[1] * 4)
    else:
        name = 'srf_vm_color_forward' if color else 'srf_vm_density_forward'

        def run():
            _lib.call(name, ctypes.byref(gs), _p(pts), p, _p(feat), _st())
        nbytes = p * (corner + 12 + feat.shape[1] * 4)
    t = _time(run, args.reps, args.warmup)
    return {'kernel': name, 'res': res, 'comps': r, 'points': p, 'ms': t * 1e3, 'gbs': nbytes / t / 1e9,
            'bytes': nbytes, 'bytes_per_point': nbytes // p}


def mlp(args):
    """Forward of the benchmark NeRF MLP (8 x 256 trunk with the skip, 128-wide view
    layer, PE degrees 10 / 4) over --m samples, 64 samples per view direction; with
    --store the training forward (the activations the backward reads are stored)."""
    from . import functional as F
    lib = _lib.load()
    prev = lib.srf_nerf_mlp_fused_path(2 if args.mlp_path == 'fused' else 0)
    spec = F.MlpSpec()
    g = torch.Generator(device='cuda').manual_seed(0)
    params = []
    for name, n in zip(spec.param_names, spec.param_numel):
        scale = 0.01 if name.endswith('bias') else 0.06
        params.append(torch.randn(n, device='cuda', generator=g) * scale)
    m, div = args.m, 64
    pts = torch.randn(m, 3, device='cuda', generator=g) * 0.7
    dirs = torch.nn.functional.normalize(torch.randn((m + div - 1) // div, 3, device='cuda', generator=g), dim=1)
    sigma = torch.empty(m, device='cuda')
    rgb = torch.empty(m, 3, device='cuda')
    prec = _lib.PRECISIONS[args.precision]
    wsb = spec.workspace_bytes(m, prec, args.store)
    ws = torch.empty(wsb, dtype=torch.uint8, device='cuda')
    scaler = torch.tensor([65536.0, 1 / 65536.0, 0.0, 0.0], device='cuda')
    arr = (ctypes.c_void_p * len(params))(*[t.data_ptr() for t in params])

    def run():
        _lib.call('srf_nerf_mlp_forward', ctypes.byref(spec.desc), arr, _p(pts), _p(dirs), div, m, None, _p(sigma),
                  _p(rgb), prec, int(args.store), _p(ws), wsb, _p(scaler), _st())
    try:
        t = _time(run, args.reps, args.warmup)
    finally:
        lib.srf_nerf_mlp_fused_path(prev)
    macs = sum(n for name, n in zip(spec.param_names, spec.param_numel) if name.endswith('weight'))
    return {'kernel': 'mlp_fused_kernel' if args.mlp_path == 'fused' else 'per-layer tc_gemm_kernel',
            'form': 'training forward (stores activations)' if args.store else 'forward only', 'm': m,
            'precision': args.precision, 'ms': t * 1e3, 'tflops': 2.0 * macs * m / t / 1e12,
            'ns_per_sample': t / m * 1e9}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('which', choices=['gemm', 'wgrad', 'composite', 'vm', 'mlp'])
    ap.add_argument('--m', type=int, default=786432)
    ap.add_argument('--k', type=int, default=256)
    ap.add_argument('--n', type=int, default=256)
    ap.add_argument('--rays', type=int, default=4096)
    ap.add_argument('--samples', type=int, default=192)
    ap.add_argument('--reps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--dgrad', action='store_true', help='gemm: backward-data epilogue (mask + column sums)')
    ap.add_argument('--backward', action='store_true', help='composite / vm: the adjoint kernel')
    ap.add_argument('--kind', choices=['color', 'density'], default='color', help='vm: which lookup')
    ap.add_argument('--res', type=int, default=300, help='vm: grid resolution per axis')
    ap.add_argument('--comps', type=int, default=48, help='vm: components per plane/line')
    ap.add_argument('--mlp-path', default='fused', choices=['fused', 'layers'], help='mlp: fused kernel or per layer')
    ap.add_argument('--store', action='store_true', help='mlp: training forward (stores the activations)')
    ap.add_argument('--precision', default='fp16', choices=['bf16', 'fp16'], help='mlp: operand format')
    args = ap.parse_args(argv)
    from . import build as _build
    _build.build()
    res = {'gemm': gemm, 'wgrad': wgrad, 'composite': composite, 'vm': vm, 'mlp': mlp}[args.which](args)
    print(json.dumps({k: (round(v, 4) if isinstance(v, float) else v) for k, v in res.items()}))


if __name__ == '__main__':
    main()
