"""Replay determinism of the captured training steps: the same CUDA graph replayed
twice from the same saved state (weights, Adam moments, step count, loss scale)
on the same batch.

Forward outputs are bit-for-bit reproducible (no kernel of the forward
accumulates with atomics).  Gradients that sum contributions with atomics (the
bias gradients of the tensor-core weight-gradient kernel, the VM scatter-add)
may differ in the last bits between replays: they are held to 1e-6 relative
(FP32 step) or 1e-4 of the largest gradient (FP16 step, loss-scaled sums), and
the bitwise-equal share is reported."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = 'cuda'


@pytest.fixture(scope='module', autouse=True)
def built():
    from simple_rf_gb300 import build as b
    b.build()


@pytest.mark.parametrize('precision', ['fp32', 'fp16'])
def test_nerf_step_replays_reproduce(precision):
    from simple_rf_gb300.train_step import NerfTrainStep, synthetic_batch
    st = NerfTrainStep(1024, 64, 128, precision=precision, device=DEV, seed=3)
    st.set_batch(*synthetic_batch(1024, 64, 128, seed=4, device=DEV))
    st.capture(warmup=1)
    torch.cuda.synchronize()
    state = [t for net in st.nets.values() for t in (net.flat, net.m, net.v)] + [st.step_count]
    if st.scaler is not None:
        state.append(st.scaler)
    saved = [t.clone() for t in state]
    runs = []
    for _ in range(2):
        for t, v in zip(state, saved):
            t.copy_(v)
        st.step()
        torch.cuda.synchronize()
        out = {k: v.clone() for k, v in st.outputs().items()}
        grads = {tag: net.grad.clone() for tag, net in st.nets.items()}
        runs.append((out, grads))
    (o1, g1), (o2, g2) = runs
    for k in o1:
        assert torch.equal(o1[k], o2[k]), k
    shares = {}
    for tag in g1:
        a, b = g1[tag].cpu().numpy(), g2[tag].cpu().numpy()
        shares[tag] = float(np.mean(a == b))
        worst = float(np.abs(a - b).max() / np.abs(a).max())
        print(precision, tag, 'largest difference between replays / largest gradient', worst)
        # FP16: the atomically summed bias gradients add loss-scaled values, whose
        # summation-order differences survive the unscaling
        bar = 1e-6 if precision == 'fp32' else 1e-4
        np.testing.assert_allclose(a, b, rtol=bar, atol=bar * float(np.abs(a).max()), err_msg=tag)
    print(precision, 'share of gradient entries bitwise equal between replays', shares)


def test_tensorf_graph_step_replays_reproduce():
    from simple_rf_gb300.bench_tensorf import make_models, synthetic_rays
    from simple_rf_gb300.tensorf_step import TensorfGraphStep
    models = make_models(DEV, precision='fp16', grids=(64, 32))
    st = TensorfGraphStep(models, 2048)
    batch = synthetic_rays(2048, 3, DEV)
    st.step(*batch)
    torch.cuda.synchronize()
    params = [p for tm in models for p in tm.parameters()]
    saved_p = [p.detach().clone() for p in params]
    saved_s = [(m.clone(), v.clone()) for m, v in st.state]
    saved_step = st.step_dev.clone()
    outs = []
    for _ in range(2):
        with torch.no_grad():
            for p, v in zip(params, saved_p):
                p.copy_(v)
            for (m, v), (sm, sv) in zip(st.state, saved_s):
                m.copy_(sm)
                v.copy_(sv)
            st.step_dev.copy_(saved_step)
        st.step(*batch)
        torch.cuda.synchronize()
        outs.append([p.detach().clone() for p in params])
    worst = 0.0
    for a, b in zip(*outs):
        d = float((a - b).abs().max())
        worst = max(worst, d / max(float(a.abs().max()), 1e-30))
    # the updated parameters differ only through the scatter-add's summation order
    assert worst < 1e-5, worst
    print('tensorf: worst relative difference of updated parameters between replays', worst)


@pytest.mark.parametrize('kind', ['density', 'color'])
def test_vm_fixed_point_scatter_is_bitwise_reproducible(kind):
    """The deterministic VM adjoint (fixed-point integer accumulation) on points
    crowded onto a few grid cells (thousands of additions per node): two runs give
    bitwise equal gradients and match the float64 oracle (grid_sample_2d_backward)
    within 1e-6 relative L2 (each contribution rounded once); the FP32-atomic
    gradients, whose long sums round at every addition, within 5e-5.  The share of
    FP32-atomic entries that differ between two runs is reported."""
    from oracle import tensorf as ot
    from simple_rf_gb300 import tensorf as T
    rng = np.random.default_rng(11)
    res = (40, 44, 48)
    comps = (16, 16, 16) if kind == 'density' else (48, 48, 48)
    planes = [(rng.standard_normal((r, res[ot.MATRIX_AXES[i][1]], res[ot.MATRIX_AXES[i][0]])) * 0.1)
              .astype(np.float32) for i, r in enumerate(comps)]
    lines = [(rng.standard_normal((r, res[ot.VECTOR_AXES[i]], 1)) * 0.1).astype(np.float32)
             for i, r in enumerate(comps)]
    n_pts = 60000
    p = rng.uniform(-1, 1, (n_pts, 3)).astype(np.float32)
    crowd = rng.random(n_pts) < 0.7                      # 70% inside one small box
    p[crowd] = rng.uniform(-0.05, 0.05, (int(crowd.sum()), 3)).astype(np.float32)
    pts = torch.from_numpy(p).to(DEV)
    if kind == 'density':
        gout = rng.standard_normal(n_pts).astype(np.float32)
    else:
        gout = rng.standard_normal((n_pts, sum(comps))).astype(np.float32)

    def grads(deterministic):
        T.set_deterministic_scatter(deterministic)
        try:
            grid = T.VmGridTensors.from_numpy(planes, lines, res, DEV)
            grid.requires_grad_(True)
            out = T.vm_density(grid, pts) if kind == 'density' else T.vm_color(grid, pts)
            (out * torch.from_numpy(gout).to(DEV)).sum().backward()
            torch.cuda.synchronize()
            return [grid.plane_grad_numpy(i) for i in range(3)] + [grid.line_grad_numpy(i) for i in range(3)]
        finally:
            T.set_deterministic_scatter(False)

    f1, f2 = grads(True), grads(True)
    a1, a2 = grads(False), grads(False)
    for x, y in zip(f1, f2):
        assert np.array_equal(x, y)
    diff = np.mean(np.concatenate([(x != y).ravel() for x, y in zip(a1, a2)]))
    feats = ot.vm_features(planes, lines, p)
    off = 0
    worst = {'fixed': 0.0, 'atomic': 0.0}
    for i in range(3):
        m0, m1 = ot.MATRIX_AXES[i]
        v = ot.VECTOR_AXES[i]
        pc, lc = feats[i]
        r = comps[i]
        d = gout[None, :].astype(np.float64) if kind == 'density' else gout[:, off:off + r].T.astype(np.float64)
        off += r
        ref_p = ot.grid_sample_2d_backward(planes[i].shape, p[:, m0], p[:, m1], d * lc, np.float64)
        ref_l = ot.grid_sample_2d_backward(lines[i].shape, np.zeros_like(p[:, v]), p[:, v], d * pc, np.float64)
        for tag, gset in (('fixed', f1), ('atomic', a1)):
            for got, ref in ((gset[i], ref_p), (gset[3 + i], ref_l)):
                worst[tag] = max(worst[tag], float(np.linalg.norm(got - ref) / np.linalg.norm(ref)))
    print(kind, 'rel-L2 vs float64', worst, 'share of FP32-atomic entries differing between runs', diff)
    assert worst['fixed'] < 1e-6 and worst['atomic'] < 5e-5, worst
