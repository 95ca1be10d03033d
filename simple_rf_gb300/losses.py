"""Drop-in loss modules whose arithmetic runs on the srf_gb300 kernels.

``TotalVariationLoss`` mirrors src/loss_functions/TotalVariationLoss04.py: the same
constructor, ``compute_loss`` contract and iteration weight, with the per-grid
squared differences and their gradients computed by ``srf_tv_loss`` (one launch
per model and grid kind).
"""
import torch

from . import functional as F


class TotalVariationLoss:
    """TotalVariationLoss04.TotalVariationLoss (TotalVariationLoss04.py:20-120)."""

    def __init__(self, configs: dict, loss_configs: dict):
        self.configs = configs
        self.loss_configs = loss_configs
        self.augmentations_needed = 'augmentations' in self.configs['model']
        self.lr_decay_ratio, self.lr_decay_iters = self.get_lr_decay_ratio_and_iters(configs)

    def get_lr_decay_ratio_and_iters(self, configs):
        """TotalVariationLoss04.py:28-37: the main optimizer's decay ratio and span."""
        lr_decay_ratio, lr_decay_iters = None, None
        for optimizer_configs in configs['optimizers']:
            if optimizer_configs['name'] == 'optimizer_main':
                lr_decay_ratio = optimizer_configs['lr_decay_ratio']
                lr_decay_iters = optimizer_configs['lr_decay_iters']
                if lr_decay_iters is None:
                    lr_decay_iters = self.configs['num_iterations']
        return lr_decay_ratio, lr_decay_iters

    def compute_loss(self, input_dict: dict, output_dict: dict, model, return_loss_maps: bool = False):
        """TotalVariationLoss04.py:39-83: TV of the density and colour grids of every
        augmented model (coarse and fine), weighted by weight_density / weight_color."""
        device = input_dict['target_rgb'].device
        total_loss = torch.zeros((), dtype=torch.float32, device=device)
        loss_maps = {}
        iter_weight = self.get_iter_weight(input_dict['iter_num'])
        if self.augmentations_needed:
            module = getattr(model, 'module', model)
            for aug_configs in self.configs['model']['augmentations']:
                aug_name = aug_configs['name']
                matches = [a for a in module.augmented_models if a['name'] == aug_name]
                if len(matches) != 1:
                    raise RuntimeError(f'expected one augmented model named {aug_name}, found {len(matches)}')
                for key in ('coarse_model', 'fine_model'):
                    if key not in aug_configs:
                        continue
                    density, color = self.get_components(matches[0][key])
                    for comps, w in ((density, self.loss_configs['weight_density']),
                                     (color, self.loss_configs['weight_color'])):
                        total_loss = total_loss + F.tv_loss(list(comps), iter_weight * w)
        loss_dict = {'loss_value': total_loss}
        if return_loss_maps:
            loss_dict['loss_maps'] = loss_maps
        return loss_dict

    @staticmethod
    def get_components(model):
        """TotalVariationLoss04.py:85-95: lines of a CP model, planes of a VM model."""
        kind = getattr(model, 'DECOMPOSITION', None) or {
            'CpDecomposedTensor': 'CandecompParafac', 'VmDecomposedTensor': 'VectorMatrix'}.get(
                model.__class__.__name__)
        if kind == 'CandecompParafac':
            return model.vectors_density, model.vectors_color
        if kind == 'VectorMatrix':
            return model.matrices_density, model.matrices_color
        raise RuntimeError(f'no TV components for {model.__class__.__name__}')

    @staticmethod
    def compute_tv_loss(components, iter_weight, return_loss_maps: bool):
        """TotalVariationLoss04.py:97-116: sum over the grids of
        2 (mean (P[h+1] - P[h])^2 + mean (P[w+1] - P[w])^2), times iter_weight."""
        loss_dict = {'loss_value': F.tv_loss(list(components), iter_weight)}
        if return_loss_maps:
            loss_dict['loss_maps'] = {}
        return loss_dict

    def get_iter_weight(self, iter_num):
        """TotalVariationLoss04.py:118-120."""
        return self.lr_decay_ratio ** ((iter_num + 1) / self.lr_decay_iters)


class _ReprojectionDepthLoss(torch.autograd.Function):
    """mean over the NeRF rays of mask2 (depth1 - depth2)^2, gradient into depth1:
    the loss AugmentationsDepthLoss11 / CoarseFineConsistencyLoss34.compute_loss_nerf
    form from their masks (their second compute_depth_mse term sees tensors the
    first zeroed in place outside mask2, and the mask rules keep mask1 & mask2
    empty).  The masks come from the reprojection kernel ``entry``; non-NeRF rays
    are masked out, and the mean runs over the NeRF rays as the reference's
    indexing by indices_mask_nerf does."""

    @staticmethod
    def forward(ctx, depth1, depth2, entry, geometry):
        rays_o, rays_d, pixel_ids, poses, k0, images, nerf_mask, patch, thr = geometry
        n = depth1.shape[0]
        d1, d2 = depth1.detach().contiguous().float(), depth2.detach().contiguous().float()
        m1 = torch.empty(n, dtype=torch.uint8, device=d1.device)
        m2 = torch.empty_like(m1)
        v, h, w, c = images.shape
        F.call(entry, F._ptr(rays_o), F._ptr(rays_d), F._ptr(d1), F._ptr(d2), F._ptr(pixel_ids), n, F._ptr(poses), v,
               F._ptr(k0), F._ptr(images), h, w, c, patch[0], patch[1], float(thr), F._ptr(m1), F._ptr(m2),
               F._stream())
        if nerf_mask is not None:
            m2 &= nerf_mask
        n_nerf = n if nerf_mask is None else int(nerf_mask.sum().item())
        loss = torch.zeros(1, device=d1.device)
        g1 = torch.zeros_like(d1)
        if n_nerf > 0:
            F.call('srf_depth_mse_loss', F._ptr(d1), F._ptr(d2), F._ptr(m2), n, float(n) / n_nerf, 0, F._ptr(loss),
                   F._ptr(g1), None, F._stream())
        ctx.save_for_backward(g1)
        ctx.mark_non_differentiable(m1, m2)
        return loss[0], m1, m2

    @staticmethod
    def backward(ctx, g_loss, _g1, _g2):
        (g1,) = ctx.saved_tensors
        # depth2 enters only as a detached target: a zero gradient, as in the reference
        g2 = torch.zeros_like(g1) if ctx.needs_input_grad[1] else None
        return g1 * g_loss, g2, None, None


class _DepthConsistencyLoss:
    """Shared geometry of the two patch-reprojection depth losses."""

    def __init__(self, configs: dict, loss_configs: dict):
        self.configs = configs
        self.loss_configs = loss_configs
        self.coarse_model_needed = 'coarse_model' in configs['model']
        self.fine_model_needed = 'fine_model' in configs['model']
        self.augmentations_needed = 'augmentations' in configs['model']
        self.patch = tuple(int(x) for x in loss_configs['patch_size'])
        self.rmse_threshold = float(loss_configs['rmse_threshold'])

    def geometry(self, input_dict, output_dict):
        dev = output_dict['rays_o'].device
        nerf = input_dict.get('indices_mask_nerf')
        nerf = None if nerf is None else nerf.to(device=dev, dtype=torch.uint8).contiguous()
        images = input_dict['common_data']['images'].to(dev).float().contiguous()
        return (output_dict['rays_o'].detach().float().contiguous(), output_dict['rays_d'].detach().float().contiguous(),
                input_dict['pixel_id'].to(dev).to(torch.int32).contiguous(),
                output_dict['extrinsics_all'].detach().float().contiguous(),
                output_dict['intrinsics'].detach()[0].float().contiguous(), images, nerf, self.patch,
                self.rmse_threshold)


class AugmentationsDepthLoss(_DepthConsistencyLoss):
    """AugmentationsDepthLoss11.AugmentationsDepthLoss (src/loss_functions/AugmentationsDepthLoss11.py:20-226):
    for each augmented model, the main model's depth is pulled towards the
    augmented depth on the rays whose reprojection into the nearest other view is
    more consistent for the augmented depth (srf_depth_reprojection_masks)."""

    def compute_loss(self, input_dict: dict, output_dict: dict, model, return_loss_maps: bool = False):
        total = torch.zeros((), device=output_dict['rays_o'].device)
        if self.augmentations_needed:
            geo = self.geometry(input_dict, output_dict)
            for tag, needed in (('coarse', self.coarse_model_needed), ('fine', self.fine_model_needed)):
                if not needed:
                    continue
                for aug in self.configs['model']['augmentations']:
                    if f'{tag}_model' in aug:
                        loss, _, _ = _ReprojectionDepthLoss.apply(
                            output_dict[f'depth_{tag}'], output_dict[f"{aug['name']}_depth_{tag}"],
                            'srf_depth_reprojection_masks', geo)
                        total = total + loss
        out = {'loss_value': total}
        if return_loss_maps:
            out['loss_maps'] = {}
        return out


class CoarseFineConsistencyLoss(_DepthConsistencyLoss):
    """CoarseFineConsistencyLoss34.CoarseFineConsistencyLoss (src/loss_functions/
    CoarseFineConsistencyLoss34.py:18-168): on the NeRF rays the coarse depth is
    pulled towards the fine depth where the fine depth reprojects more
    consistently (srf_coarse_fine_reprojection_masks); on the sparse-depth rays the
    coarse depth is pulled towards the fine depth (compute_loss_sd)."""

    def __init__(self, configs: dict, loss_configs: dict):
        super().__init__(configs, loss_configs)
        self.sparse_depth_needed = 'sparse_depth' in configs['data_loader']

    def compute_loss(self, input_dict: dict, output_dict: dict, model, return_loss_maps: bool = False):
        total = torch.zeros((), device=output_dict['rays_o'].device)
        if self.coarse_model_needed and self.fine_model_needed:
            geo = self.geometry(input_dict, output_dict)
            loss, _, _ = _ReprojectionDepthLoss.apply(output_dict['depth_coarse'], output_dict['depth_fine'],
                                                      'srf_coarse_fine_reprojection_masks', geo)
            total = total + loss
            sd = input_dict.get('indices_mask_sparse_depth')
            if self.sparse_depth_needed and sd is not None:
                total = total + F.depth_mse(output_dict['depth_coarse'], output_dict['depth_fine'].detach(),
                                            sd.to(output_dict['rays_o'].device))
        out = {'loss_value': total}
        if return_loss_maps:
            out['loss_maps'] = {}
        return out
