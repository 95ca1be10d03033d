"""TensoRF VM training-step workload: a 300^3 main model and a 75^3 augmented
model forward + backward + Adam on the srf_gb300 kernels, through the drop-in
``GbVmTensor`` modules (the path ``SimpleTensoRF.render_rays`` drives,
src/models/SimpleTensoRF09.py:194-351 and LowRankTensor.forward :701-761).

Workload (per step): 8192 rays; bbox [-1.5, 1.5]^3; density 16 components per
plane/line, appearance 48 per plane/line projected to 27 features; renderer
PE L=2 on features and view direction -> 128 -> 128 -> 3; planes/lines ~
N(0, 0.1^2); ReLU density, distance scale 25; sample step half a voxel (1039
samples per ray at 300^3, 260 at 75^3); a 128^3 alpha-mask volume with
Bernoulli(0.15) occupancy (trilinear lookup > 0, so a sample is kept when any of
its 8 neighbouring cells is occupied).  Rays: origins uniform on the sphere of
radius 4 about the box centre, directions towards the centre perturbed by
N(0, 0.3^2) per axis, near 2, far 6.  Loss: MSE of each model's rgb against
targets ~ U[0,1]^3.

    python -m simple_rf_gb300.bench_tensorf --rays 8192 --steps 10 --warmup 3 [--precision fp16] [--eager]
    python -m simple_rf_gb300.bench_tensorf --sweep        # ray batches 1024 ... 65536
    python -m simple_rf_gb300.bench_tensorf --renderer-rows 1200000 --steps 5 [--forward-only] [--adjoint simt]
"""
import argparse
import json

import torch

from . import _lib
from . import functional as F
from .tensorf_step import TensorfGraphStep, TensorfTrainStep

BBOX = [[-1.5] * 3, [1.5] * 3]


def tensor_configs(n_voxels):
    return {'decomposition_type': 'VectorMatrix', 'num_samples_max': 1e6, 'num_components_density': [16, 16, 16],
            'num_components_color': [48, 48, 48], 'bounding_box': BBOX, 'num_voxels_initial': n_voxels,
            'num_voxels_final': n_voxels, 'tensor_upsampling_iters': [], 'num_voxels_per_sample': 0.5,
            'alpha_mask_update_iters': [], 'alpha_mask_threshold': 1e-4, 'ray_marching_weight_threshold': 1e-4,
            'use_view_dirs': True, 'view_dependent_color': True, 'views_positional_encoding_degree': 2,
            'features_positional_encoding_degree': 2, 'features_dimension_color': 27, 'density_offset': -10,
            'distance_scale': 25, 'density_predictor': 'ReLU', 'color_predictor': 'MLP_Features',
            'num_units_color_predictor': 128, 'predict_visibility': False}


def make_models(device, seed=0, mask_res=128, mask_occupancy=0.15, precision='fp32', grids=(300, 75)):
    from .tensorf_model import AlphaGridMask, GbVmTensor
    torch.manual_seed(seed)
    configs = {'data_loader': {'ndc': False}, 'model': {'white_bkgd': True, 'precision': precision}}
    models = []
    for name, nv in (('coarse_model', grids[0] ** 3), ('views_augmentation_coarse_model', grids[1] ** 3)):
        tm = GbVmTensor(name, configs, tensor_configs(nv), {'bounding_box': BBOX}).to(device)
        g = torch.Generator().manual_seed(seed + 1)
        vol = (torch.rand(mask_res, mask_res, mask_res, generator=g) < mask_occupancy).to(device)
        tm.alpha_mask = AlphaGridMask(vol, tm.bounding_box.detach().clone())
        models.append(tm)
    return models


def synthetic_rays(n, seed, device):
    g = torch.Generator().manual_seed(seed)
    o = torch.randn(n, 3, generator=g)
    o = 4.0 * o / torch.linalg.norm(o, dim=-1, keepdim=True)
    d = -o / 4.0 + 0.3 * torch.randn(n, 3, generator=g)
    d = d / torch.linalg.norm(d, dim=-1, keepdim=True)
    t_rgb = torch.rand(n, 3, generator=g)
    u = torch.rand(n, 2, generator=g)
    return [x.to(device) for x in (o, d, t_rgb, u)]


SWEEP_RAYS = (1024, 2048, 4096, 8192, 16384, 32768, 65536)


def ray_batch_sweep(device, modes=(('fp16', False), ('fp16', True), ('fp32', False)), sizes=SWEEP_RAYS, warmup=2,
                    steps=3, seed=0):
    """Train rays/s of the same step over ray batches of 1024 ... 65536 rays: one model
    pair per (precision, captured-or-not) mode, trained on from size to size (each size
    gets its own warm-up, and its own CUDA graph when captured), rays drawn afresh per
    size.  Keys: 'fp16' / 'fp32' (uncaptured, one host read of the sample counts per
    phase), 'fp16_graph' (TensorfGraphStep)."""
    out = {}
    for prec, graph in modes:
        models = make_models(device, seed=seed, precision=prec)
        eager = None if graph else TensorfTrainStep(models)
        state = step_dev = None
        res = {}
        for n in sizes:
            if graph:
                # Adam state and step count carry over from size to size
                st = TensorfGraphStep(models, n, state=state, step_dev=step_dev)
                state, step_dev = st.state, st.step_dev
            else:
                st = eager
            batches = [synthetic_rays(n, 100 + i, device) for i in range(2)]
            for i in range(warmup):
                st.step(*batches[i % 2])
            torch.cuda.synchronize(device)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for i in range(steps):
                st.step(*batches[i % 2])
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1) / steps
            surf = st.sample_counts()[0]['surface'] if graph else st.last['samples'][0]['surface']
            res[str(n)] = {'ms_per_step': round(ms, 3), 'rays_per_s': round(n / ms * 1e3, 1),
                           'surface_samples': int(surf)}
            if graph:
                res[str(n)]['recaptures'] = st.recaptures
                res[str(n)]['capacity_shrinks'] = st.shrinks
                del st
            del batches
            torch.cuda.empty_cache()
        out[prec + ('_graph' if graph else '')] = res
        del models, eager, state, step_dev
        torch.cuda.empty_cache()
    for key in ('fp16', 'fp16_graph'):
        if key in out and 'fp32' in out:
            out[f'speedup_{key}_vs_fp32_plain'] = {n: round(out[key][n]['rays_per_s'] / out['fp32'][n]['rays_per_s'], 2)
                                                   for n in out[key]}
    return out


def renderer_case(dev, rows, reps=5, adjoint='tc', backward=True):
    """The FP16 tensor-core renderer (basis 144 -> 27 + PE + 128 -> 128 -> 3) alone on
    ``rows`` synthetic surface samples (features ~ N(0, 0.3^2), unit view
    directions): forward and (``backward``) backward ``reps`` times after three
    warm-up passes; ``adjoint`` picks the basis adjoint ('tc' or 'simt')."""
    from . import tensorf as T
    tm = make_models(dev, precision='fp16', grids=(64, 32))[0]
    cp = tm.color_predictor
    g = torch.Generator(device=dev).manual_seed(0)
    feats = (torch.randn(rows, 144, device=dev, generator=g) * 0.3).requires_grad_(backward)
    vd = torch.nn.functional.normalize(torch.randn(rows, 3, device=dev, generator=g), dim=-1)
    d_rgb = torch.rand(rows, 3, device=dev, generator=g)
    desc = _lib.RendererDesc(144, cp.features_dimension, cp.mlp[0].out_features, cp.lf, cp.lv, 1)
    params = [tm.basis_matrix_color.weight, cp.mlp[0].weight, cp.mlp[0].bias, cp.mlp[2].weight, cp.mlp[2].bias,
              cp.mlp[4].weight, cp.mlp[4].bias]
    _lib.check(_lib.load().srf_tensorf_basis_adjoint_path(int(adjoint == 'tc')), 'srf_tensorf_basis_adjoint_path')

    def once():
        with torch.set_grad_enabled(backward):
            rgb = T.renderer_tc(desc, _lib.SRF_PRECISION_FP16, feats, vd, params)
            if backward:
                rgb.backward(d_rgb)

    for _ in range(3):
        once()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.profiler.start()
    e0.record()
    for _ in range(reps):
        once()
    e1.record()
    torch.cuda.profiler.stop()
    e1.synchronize()
    return {'workload': f'tensorf_renderer_fp16_{rows}rows', 'rows': rows, 'backward': backward, 'adjoint': adjoint,
            'ms_per_pass': round(e0.elapsed_time(e1) / reps, 4)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('--rays', type=int, default=8192)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--precision', default='fp32', choices=['fp32', 'bf16', 'fp16'],
                    help='renderer MLP: FP32 SIMT or 16-bit tensor cores')
    ap.add_argument('--sweep', action='store_true', help='ray-batch sweep 1024 ... 65536, FP16 and FP32 plain')
    ap.add_argument('--eager', action='store_true', help='the uncaptured step (host reads of the sample counts)')
    ap.add_argument('--renderer-rows', type=int, default=0,
                    help='time the FP16 renderer alone (forward + backward) on this many surface samples')
    ap.add_argument('--forward-only', action='store_true', help='with --renderer-rows: the forward alone')
    ap.add_argument('--adjoint', default='tc', choices=['tc', 'simt'], help='with --renderer-rows: basis adjoint')
    ap.add_argument('--deterministic', action='store_true',
                    help='VM grid adjoints through the fixed-point (bitwise reproducible) scatter-add')
    args = ap.parse_args(argv)
    from . import build as _build
    _build.build()
    dev = torch.device('cuda')
    if args.renderer_rows:
        print(json.dumps(renderer_case(dev, args.renderer_rows, reps=args.steps, adjoint=args.adjoint,
                                       backward=not args.forward_only)))
        return
    if args.sweep:
        print(json.dumps({'workload': 'tensorf_vm_train_step_ray_batch_sweep_300^3+75^3',
                          'sweep': ray_batch_sweep(dev)}))
        return
    if args.deterministic:
        from . import tensorf as T
        T.set_deterministic_scatter(True)
    models = make_models(dev, precision=args.precision)
    step = TensorfTrainStep(models) if args.eager else TensorfGraphStep(models, args.rays)
    batches = [synthetic_rays(args.rays, 10 + i, dev) for i in range(4)]
    for i in range(args.warmup):
        step.step(*batches[i % 4])
    torch.cuda.synchronize()
    lib = _lib.load()
    l0 = lib.srf_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    # the timed steps are the range a profiler started with profiling off captures
    torch.cuda.profiler.start()
    with F.nvtx_range('srf.timed_steps'):
        for i in range(args.steps):
            step.step(*batches[i % 4])
    e1.record()
    torch.cuda.profiler.stop()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / max(args.steps, 1)
    if args.eager:
        launches = (lib.srf_launch_count() - l0) / max(args.steps, 1)
        samples, loss = step.last['samples'], step.last['loss']
    else:
        launches, samples, loss = step.launches_per_step, step.sample_counts(), step.loss
    print(json.dumps({'workload': f'tensorf_vm_train_step_{args.rays}rays_300^3+75^3', 'rays': args.rays,
                      'precision': args.precision, 'cuda_graph': not args.eager,
                      'deterministic_scatter': args.deterministic,
                      'ms_per_step': round(ms, 4), 'rays_per_s': round(args.rays / ms * 1e3, 1),
                      'samples_per_step': {m.name: c for m, c in zip(models, samples)},
                      'gpu_launches_per_step': launches, 'loss': float(loss.item())}))


if __name__ == '__main__':
    main()
