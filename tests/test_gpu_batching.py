"""Device-side batch assembly (srf_batch_assemble, simple_rf_gb300.batching) for
cached-ray training, the counterpart of DataPreprocessor10.select_batch_indices /
load_nerf_cached_batch / load_sparse_depth_cached_batch
(src/data_preprocessors/DataPreprocessor10.py:496-594): the order matches its host
restatement, epochs visit distinct rays, the gathers are exact, the batch
dictionary has the reference's keys and -1 fills, and a captured training step
that draws its own batches equals the eager step fed the same batch."""
import numpy as np
import pytest
import torch

from test_batching_host import batch_indices

pytestmark = pytest.mark.gpu
DEV = 'cuda'


@pytest.fixture(scope='module', autouse=True)
def built():
    from simple_rf_gb300 import build as b
    b.build()


def _pool(p=10000, views=5, h=60, w=80, seed=0):
    g = torch.Generator().manual_seed(seed)
    pid = torch.stack([torch.randint(0, views, (p,), generator=g), torch.randint(0, w, (p,), generator=g),
                       torch.randint(0, h, (p,), generator=g)], 1).int()
    rgb = torch.rand(p, 3, generator=g)
    intr = torch.tensor([[60.0, 0, w / 2], [0, 60.0, h / 2], [0, 0, 1]]).repeat(views, 1, 1)
    extr = torch.eye(4).repeat(views, 1, 1)
    extr[:, :3, 3] = torch.randn(views, 3, generator=g) * 0.1
    return pid, rgb, intr, extr


def test_batches_follow_the_order_and_gather_exactly():
    from simple_rf_gb300.batching import GpuRayBatcher
    pid, rgb, intr, extr = _pool()
    n = 4096
    bt = GpuRayBatcher(pid, rgb, n, intrinsics=intr, extrinsics=extr, seed=12345)
    seen = []
    for step in range(6):   # 3 epochs of 2 full batches
        batch = bt.get_next_batch(step)
        idx = batch['indices'].cpu().numpy().astype(np.int64)
        assert idx.tolist() == batch_indices(10000, n, 12345, step)
        np.testing.assert_array_equal(batch['pixel_id'].cpu().numpy(), pid.numpy()[idx])
        np.testing.assert_array_equal(batch['target_rgb'].cpu().numpy(), rgb.numpy()[idx])
        img = pid.numpy()[idx, 0]
        np.testing.assert_array_equal(batch['intrinsics'].cpu().numpy(), intr.numpy()[img])
        np.testing.assert_array_equal(batch['extrinsics'].cpu().numpy(), extr.numpy()[img])
        assert batch['indices_mask_nerf'].all() and batch['num_frames'] == 5 and batch['iter_num'] == step
        seen.append(idx)
    for e in range(3):
        ep = np.concatenate(seen[2 * e:2 * e + 2])
        assert len(np.unique(ep)) == 2 * n
    assert not np.array_equal(seen[0], seen[2])
    from simple_rf_gb300 import _lib
    import ctypes
    fl = ctypes.c_int(0)
    _lib.check(_lib.load().srf_read_device_flag(ctypes.byref(fl), None), 'flag')
    assert fl.value == 0


def test_sparse_depth_rows_follow_the_reference_layout():
    from simple_rf_gb300.batching import GpuRayBatcher
    pid, rgb, intr, extr = _pool(p=3000)
    g = torch.Generator().manual_seed(4)
    sd_idx = torch.randperm(3000, generator=g)[:700]
    depths = torch.full((3000,), -5.0)
    depths[sd_idx] = torch.rand(700, generator=g) * 4 + 1
    errs = torch.rand(3000, generator=g)
    pts = torch.randn(3000, 3, generator=g)
    bt = GpuRayBatcher(pid, rgb, 1024, seed=1, sparse_depth={'indices': sd_idx, 'depths': depths,
                                                           'reprojection_errors': errs, 'points_3d': pts},
                       num_rays_sparse_depth=256)
    b = bt.get_next_batch(0)
    n, m = 1024, 256
    assert b['pixel_id'].shape == (n + m, 3)
    mn, ms = b['indices_mask_nerf'].cpu().numpy(), b['indices_mask_sparse_depth'].cpu().numpy()
    assert mn[:n].all() and not mn[n:].any() and ms[n:].all() and not ms[:n].any()
    idx = b['indices'].cpu().numpy().astype(np.int64)
    assert set(idx[n:].tolist()) <= set(sd_idx.tolist()) and len(set(idx[n:].tolist())) == m
    np.testing.assert_array_equal(b['pixel_id'].cpu().numpy(), pid.numpy()[idx])
    np.testing.assert_array_equal(b['target_rgb'].cpu().numpy()[n:], -np.ones((m, 3), np.float32))
    np.testing.assert_array_equal(b['sparse_depth_values'].cpu().numpy()[n:, 0], depths.numpy()[idx[n:]])
    np.testing.assert_array_equal(b['sparse_depth_values'].cpu().numpy()[:n], -np.ones((n, 1), np.float32))
    np.testing.assert_array_equal(b['sparse_depth_errors'].cpu().numpy()[n:, 0], errs.numpy()[idx[n:]])
    np.testing.assert_array_equal(b['sparse_depth_points3d'].cpu().numpy()[n:], pts.numpy()[idx[n:]])


def test_counter_uniforms():
    from simple_rf_gb300 import _lib
    from simple_rf_gb300.functional import _ptr, _stream
    c = torch.zeros(1, dtype=torch.int32, device=DEV)
    u = [torch.empty(1 << 20, device=DEV) for _ in range(3)]
    _lib.call('srf_uniforms', _ptr(u[0]), u[0].numel(), 9, _ptr(c), 0, _stream())
    _lib.call('srf_uniforms', _ptr(u[1]), u[1].numel(), 9, _ptr(c), 0, _stream())
    c += 1
    _lib.call('srf_uniforms', _ptr(u[2]), u[2].numel(), 9, _ptr(c), 0, _stream())
    assert torch.equal(u[0], u[1]) and not torch.equal(u[0], u[2])
    for x in u:
        assert float(x.min()) >= 0.0 and float(x.max()) < 1.0
        assert abs(float(x.mean()) - 0.5) < 2e-3 and abs(float(x.var()) - 1 / 12) < 2e-3


def test_captured_step_with_device_batches_equals_eager_step():
    """A captured FP32 step that assembles its batch (pixel rays, uniforms) on the
    device equals an eager step fed that batch through set_batch."""
    from simple_rf_gb300 import _lib, functional as F
    from simple_rf_gb300.batching import GpuRayBatcher
    from simple_rf_gb300.train_step import NerfTrainStep
    pid, rgb, intr, extr = _pool(p=2000)
    n = 256
    a = NerfTrainStep(n, 64, 128, precision='fp32', device=DEV, seed=5, depth_fraction=0.0)
    bt = GpuRayBatcher(pid, rgb, n, intrinsics=intr, extrinsics=extr, seed=77)
    a.attach_batcher(bt, seed=99)
    a.capture(warmup=0)
    ref = NerfTrainStep(n, 64, 128, precision='fp32', device=DEV, seed=5, depth_fraction=0.0)
    for step in range(3):
        # the batch the captured step will draw at this counter value
        o = bt.assemble()
        ro, rd = F.pixel_rays(o['pixel_id'], o['intrinsics'], o['extrinsics'])
        u_c, u_f = torch.empty(n, 64, device=DEV), torch.empty(n, 128, device=DEV)
        for sid, u in enumerate((u_c, u_f)):
            _lib.call('srf_uniforms', F._ptr(u), u.numel(), 99, F._ptr(bt.counter), sid, F._stream())
        ref.set_batch(ro, rd, o['target_rgb'].clone(), torch.zeros(n, device=DEV), u_c, u_f)
        ref.step()
        a.step()
        torch.cuda.synchronize()
        assert int(bt.counter.item()) == step + 1
        # every step's inputs are the batch of its counter value, bit for bit
        for mine, theirs in ((a.rays_o, ro), (a.rays_d, rd), (a.target_rgb, o['target_rgb']), (a.u_c, u_c),
                             (a.u_f, u_f)):
            assert torch.equal(mine, theirs), step
        # the first step starts from equal weights and matches bit for bit (later
        # steps start from weights that Adam moved by +-lr wherever the atomically
        # summed gradients differ in sign, so they are not compared)
        if step == 0:
            for k in ('rgb_map', 'depth', 'weights'):
                for tag in ('coarse', 'fine'):
                    assert torch.equal(a.buf[tag][k], ref.buf[tag][k]), (step, k, tag)
