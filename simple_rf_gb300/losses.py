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
