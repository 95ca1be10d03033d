"""Cached-ray training batches assembled on the device.

``GpuRayBatcher`` replaces the batching mode of DataPreprocessor10.get_next_batch
(src/data_preprocessors/DataPreprocessor10.py:450-549: select_batch_indices,
load_nerf_cached_batch and load_sparse_depth_cached_batch): every epoch visits
the cached rays in a fresh random order in consecutive slices of ``num_rays``,
optionally followed by ``num_rays_sparse_depth`` sparse-depth rays drawn the
same way from the sparse-depth pixels, and returns the same batch dictionary
keys (``indices``, ``indices_mask_nerf``, ``pixel_id``, ``target_rgb``,
``indices_mask_sparse_depth``, ``sparse_depth_values`` ...), with -1 in the rows
a part does not fill, as the reference does.

The reference shuffles a host numpy index array and copies each batch to the
device; here the order is a keyed bijection evaluated by the srf_batch_assemble
kernel and the batch counter lives on the device, so the whole training
iteration (batch, rays, render, loss, backward, update) can be one CUDA graph.
The random order differs from numpy's (no implementation shares a random
stream with numpy's shuffle); each epoch still visits every cached ray once,
except the ``pool mod num_rays`` rays an epoch leaves over, which the
reference would put in a shorter last batch.
"""
import torch

from . import _lib
from .functional import _ptr, _stream


class GpuRayBatcher:
    def __init__(self, pixel_id, target_rgb, num_rays, *, intrinsics=None, extrinsics=None, seed=0, device='cuda',
                 sparse_depth=None, num_rays_sparse_depth=0):
        """pixel_id (P,3) (image, x, y), target_rgb (P,3): the cached rays.
        intrinsics (V,3,3) / extrinsics (V,4,4): optional cameras, gathered per ray
        for srf_pixel_rays.  sparse_depth: optional dict with 'indices' (the pixel
        indices that carry a sparse depth), and full-size (P,) 'depths',
        'reprojection_errors' and (P,3) 'points_3d' as the reference's
        sparse_depth_data holds them."""
        dev = torch.device(device)
        self.device = dev
        self.num_rays = int(num_rays)
        self.seed = int(seed) & ((1 << 64) - 1)
        self.pool_pid = torch.as_tensor(pixel_id).to(dev, torch.int32).contiguous()
        self.pool_rgb = torch.as_tensor(target_rgb).to(dev, torch.float32).contiguous()
        p = self.pool_pid.shape[0]
        if self.pool_rgb.shape != (p, 3) or self.pool_pid.shape != (p, 3):
            raise ValueError('pixel_id and target_rgb must be (P, 3)')
        if p < self.num_rays:
            raise ValueError(f'{p} cached rays cannot fill batches of {self.num_rays}')
        self.num_frames = int(self.pool_pid[:, 0].max().item()) + 1 if p else 0
        self.intr = None if intrinsics is None else torch.as_tensor(intrinsics).to(dev, torch.float32).contiguous()
        self.extr = None if extrinsics is None else torch.as_tensor(extrinsics).to(dev, torch.float32).contiguous()
        self.n_views = 0 if self.extr is None and self.intr is None else \
            int((self.extr if self.extr is not None else self.intr).shape[0])
        self.nsd = int(num_rays_sparse_depth) if sparse_depth is not None else 0
        n = self.num_rays + self.nsd
        self.counter = torch.zeros(1, dtype=torch.int32, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        self.out = {'indices': torch.empty(n, **i32), 'pixel_id': torch.full((n, 3), -1, **i32),
                    'target_rgb': torch.full((n, 3), -1.0, device=dev)}
        mask = torch.zeros(n, dtype=torch.bool, device=dev)
        mask[:self.num_rays] = True
        self.out['indices_mask_nerf'] = mask
        if self.intr is not None:
            self.out['intrinsics'] = torch.zeros(n, 3, 3, device=dev)
        if self.extr is not None:
            self.out['extrinsics'] = torch.zeros(n, 4, 4, device=dev)
        if self.nsd:
            sd = sparse_depth
            self.sd_rows = torch.as_tensor(sd['indices']).to(dev, torch.int32).contiguous()
            if self.sd_rows.numel() < self.nsd:
                raise ValueError('fewer sparse-depth pixels than sparse-depth rays per batch')
            vals = torch.full((p, 5), -1.0, device=dev)
            vals[:, 0] = torch.as_tensor(sd['depths']).to(dev, torch.float32).reshape(p)
            vals[:, 1] = torch.as_tensor(sd['reprojection_errors']).to(dev, torch.float32).reshape(p)
            vals[:, 2:5] = torch.as_tensor(sd['points_3d']).to(dev, torch.float32).reshape(p, 3)
            self.sd_values = vals.contiguous()
            self.sd_out = torch.full((self.nsd, 5), -1.0, device=dev)
            self.out['indices_mask_sparse_depth'] = ~mask
            for k in ('sparse_depth_values', 'sparse_depth_errors'):
                self.out[k] = torch.full((n, 1), -1.0, device=dev)
            self.out['sparse_depth_points3d'] = torch.full((n, 3), -1.0, device=dev)

    def assemble(self):
        """Enqueue the gathers of the current batch (the counter is not advanced)."""
        st = _stream()
        o = self.out
        n = self.num_rays
        rows = self.pool_pid.shape[0]
        _lib.call('srf_batch_assemble', None, _ptr(self.pool_pid), _ptr(self.pool_rgb), 3, rows, rows, n,
                  self.seed, _ptr(self.counter), _ptr(self.intr), _ptr(self.extr), self.n_views, _ptr(o['pixel_id']),
                  _ptr(o['target_rgb']), _ptr(o['indices']), _ptr(o.get('intrinsics')), _ptr(o.get('extrinsics')), st)
        if self.nsd:
            m = self.nsd
            # a second, independently keyed order over the sparse-depth pixels; rows [n, n + m)
            pid_tail = o['pixel_id'][n:]
            intr_tail = o['intrinsics'][n:] if 'intrinsics' in o else None
            extr_tail = o['extrinsics'][n:] if 'extrinsics' in o else None
            _lib.call('srf_batch_assemble', _ptr(self.sd_rows), _ptr(self.pool_pid), _ptr(self.sd_values), 5,
                      self.sd_rows.numel(), rows, m, (self.seed ^ 0x5D5D5D5D5D5D5D5D) & ((1 << 64) - 1),
                      _ptr(self.counter), _ptr(self.intr), _ptr(self.extr), self.n_views, _ptr(pid_tail),
                      _ptr(self.sd_out), _ptr(o['indices'][n:]), _ptr(intr_tail), _ptr(extr_tail), st)
            o['sparse_depth_values'][n:, 0].copy_(self.sd_out[:, 0])
            o['sparse_depth_errors'][n:, 0].copy_(self.sd_out[:, 1])
            o['sparse_depth_points3d'][n:].copy_(self.sd_out[:, 2:5])
        return o

    def advance(self):
        """Enqueue the counter increment (the next assemble() takes the next batch)."""
        _lib.call('srf_counter_add', _ptr(self.counter), 1, None, _stream())

    def get_next_batch(self, iter_num: int, image_num: int = None):
        """DataPreprocessor10.get_next_batch in batching mode (image_num None): the
        batch dictionary of the next cached batch; the tensors are the batcher's
        own buffers, refilled by the next call."""
        if image_num is not None:
            raise NotImplementedError('whole-image batches are served by the host data pipeline')
        self.assemble()
        self.advance()
        batch = dict(self.out)
        batch['iter_num'] = iter_num
        batch['num_frames'] = self.num_frames
        batch['common_data'] = {}
        return batch
