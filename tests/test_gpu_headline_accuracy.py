"""The benchmark's headline training step (FP16 operands on the tcgen05 tensor
cores, FP32 accumulation, FP32 master weights, FP32 PE and compositing, dynamic
loss scale) at its full 4096 rays against the float64 oracle.

Bars of the metric: rendered rgb within 2e-3 max-abs, parameter gradients within
1e-2 relative L2 (whole gradient of each net).

* rgb: the Xavier-initialised nets of the benchmark, every one of the 4096 rays,
  coarse and fine (the fine pass on the depths the GPU sampled).  A ray whose
  last-sample raw sigma is zero on one side and positive on the other (the
  delta = 1e10 |d| step of SimpleNeRF17.py:489-492) switches between the white
  background and that sample's colour; such rays are counted, must stay below
  0.5% of the batch, and are the only ones left out.
* gradients: 1024 rays of the same step on a network whose sigma-head bias (0.5)
  keeps every ray off that step (see test_gpu_train_step.py).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
HEADLINE = 'fp16'


@pytest.fixture(scope='module', autouse=True)
def built():
    from simple_rf_gb300 import build as b
    b.build()


def test_headline_step_rgb_on_4096_rays_against_fp64_oracle():
    from test_gpu_benchmark_workloads import _step, oracle_step_chunked
    params, out, _, host = _step(4096, precision=HEADLINE, seed=7)
    ref, _ = oracle_step_chunked(params, host, out['z_fine'], np.float64, chunk=512, grads=False)
    flip = np.zeros(4096, bool)
    for tag in ('coarse', 'fine'):
        flip |= (out[f'sigma_{tag}'].reshape(4096, -1)[:, -1] > 0) != (ref[f'raw_sigma_{tag}'][:, -1, 0] > 0)
    assert flip.mean() < 0.005, int(flip.sum())
    worst = {}
    for tag in ('coarse', 'fine'):
        err = np.abs(out[f'rgb_map_{tag}'] - ref[f'rgb_{tag}']).max(1)
        worst[tag] = float(err[~flip].max())
        assert worst[tag] < 2e-3, (tag, worst[tag])
    print(f'{HEADLINE} step, 4096 rays: rgb max-abs vs float64 {worst}; rays with a last-sample flip '
          f'{int(flip.sum())}')


def test_headline_step_gradients_against_fp64_oracle():
    """Whole-gradient relative L2 of each net on 1024 rays.  A ray whose last-sample
    sigma flips between zero and positive has a gradient of order 1e10 in either
    implementation, so the comparison needs a batch with none: the first of five
    seeded batches whose 1024 rays have no flip against the float64 oracle is
    used (the step is deterministic, so the choice is fixed), and the flips of
    the rejected batches are reported."""
    from test_gpu_benchmark_workloads import _step, oracle_step_chunked
    rejected = {}
    for seed in range(7, 12):
        params, out, grads, host = _step(1024, precision=HEADLINE, sigma_bias=0.5, seed=seed)
        ref, _ = oracle_step_chunked(params, host, out['z_fine'], np.float64, chunk=256, grads=False)
        flips = 0
        for tag in ('coarse', 'fine'):
            flips += int(((out[f'sigma_{tag}'].reshape(1024, -1)[:, -1] > 0) !=
                          (ref[f'raw_sigma_{tag}'][:, -1, 0] > 0)).sum())
        if flips == 0:
            break
        rejected[seed] = flips
    assert flips == 0, rejected
    ref, g64 = oracle_step_chunked(params, host, out['z_fine'], np.float64, chunk=256)
    for tag in ('coarse', 'fine'):
        err = np.abs(out[f'rgb_map_{tag}'] - ref[f'rgb_{tag}']).max()
        assert err < 2e-3, (tag, err)
        got = np.concatenate([grads[tag][k].ravel() for k in g64[tag]])
        want = np.concatenate([g64[tag][k].ravel() for k in g64[tag]])
        rel = np.linalg.norm(got - want) / np.linalg.norm(want)
        print(f'{HEADLINE} step, 1024 rays (seed {seed}, batches rejected for a flip: {rejected}), {tag}: '
              f'whole-gradient rel-L2 {rel:.4g}, rgb max-abs {err:.3g}')
        assert rel < 1e-2, (tag, rel)
