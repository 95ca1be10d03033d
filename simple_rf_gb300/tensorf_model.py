"""Drop-in Simple-TensoRF model running on the srf_gb300 CUDA kernels.

``GbSimpleTensoRF(configs, model_configs)`` mirrors ``SimpleTensoRF``
(src/models/SimpleTensoRF09.py:16-544) with the VM decomposition
(``VmDecomposedTensor`` :1126-1320): same constructor, forward contract, output
keys, buffer/parameter names and logical shapes.  The render path runs on the
hand-written kernels: ray generation, AABB ray marching or stratified NDC
samples, bbox + alpha-mask validity with stream compaction of the uneven
per-ray sample lists, VM density/colour gathers from channels-last planes, the
basis + renderer MLP, and compositing; the backward passes are the adjoint
kernels (VM gradients are scatter-adds).

Training-time maintenance (alpha-mask rebuild, bbox shrink, grid upsampling,
optimizer surgery; SimpleTensoRF09.py:821-944) runs every few thousand
iterations and is written with torch tensor ops on the channels-last views,
with the dense density evaluation on the VM density kernel.  The CP
decomposition (``CpDecomposedTensor``, SimpleTensoRF09.py:964-1123) is
``GbCpTensor``: three lines per density/colour tensor on the CP lookup kernels.
"""
import weakref

import numpy
import torch
from torch.nn import ModuleDict, ModuleList

from . import _lib
from . import functional as F
from . import tensorf as T
from .nerf import ExtrinsicsLearner, IntrinsicsLearner, _precision, check_pose_learning

MATRIX_AXES = [[0, 1], [0, 2], [1, 2]]   # SimpleTensoRF09.py:1131
VECTOR_AXES = [2, 1, 0]                  # SimpleTensoRF09.py:1132


def compute_resolution_in_voxels(num_voxels, bounding_box):
    """SimpleTensoRF09.py:625-638: cubic voxels filling the box."""
    lo, hi = bounding_box
    size = ((hi - lo).prod() / num_voxels).pow(1 / len(lo))
    return ((hi - lo) / size).long()


def cached_host(owner, tag, t):
    """The values of tensor ``t`` as a host list, re-read (one device sync) only when
    ``t`` is a different tensor object or was modified in place since the last read:
    the model's geometry buffers change only when the grid is resized or loaded."""
    cache = owner.__dict__.setdefault('_host_cache', {})
    hit = cache.get(tag)
    if hit is not None and hit[0]() is t and hit[1] == t._version:
        return hit[2]
    val = t.detach().cpu().reshape(-1).tolist()
    cache[tag] = (weakref.ref(t), t._version, val)
    return val


class AlphaGridMask(torch.nn.Module):
    """Occupancy volume (SimpleTensoRF09.py:1323-1367); state saved as bool, used as float."""

    def __init__(self, alpha_volume, bounding_box):
        super().__init__()
        self.register_buffer('alpha_volume', torch.tensor(0, dtype=torch.bool))
        self.register_buffer('bounding_box', torch.zeros(2, 3))
        self.register_buffer('bounding_box_size', torch.zeros(3))
        self.register_buffer('resolution', torch.zeros(3, dtype=torch.long))
        self.alpha_volume = alpha_volume.float().view(1, 1, *alpha_volume.shape[-3:])
        self.bounding_box = bounding_box
        self.bounding_box_size = self.bounding_box[1] - self.bounding_box[0]
        d, h, w = alpha_volume.shape[-3:]
        self.resolution = torch.tensor([w, h, d], dtype=torch.long, device=alpha_volume.device)
        self._register_state_dict_hook(lambda mod, sd, prefix, *a: sd.__setitem__(
            f'{prefix}alpha_volume', sd[f'{prefix}alpha_volume'].bool()))
        self._register_load_state_dict_pre_hook(self._load_hook)

    @staticmethod
    def _load_hook(sd, prefix, *args, **kwargs):
        sd[f'{prefix}alpha_volume'] = sd[f'{prefix}alpha_volume'].float()

    def volume(self):
        return self.alpha_volume.reshape(self.alpha_volume.shape[-3:]).contiguous().float()

    def sample_alpha(self, pts):
        """Positive/zero occupancy (as float) of world points (:1342-1345 followed by > 0)."""
        pn = ((pts - self.bounding_box[0]) / self.bounding_box_size) * 2 - 1
        return T.alpha_mask_query(self.volume(), pn.reshape(-1, 3).contiguous().float()).float()


class MlpFeaturesColorPredictor(torch.nn.Module):
    """SimpleTensoRF09.py:1370-1421: PE(features) + PE(view dirs) -> 128 -> 128 -> 3."""

    def __init__(self, tensor_configs, features_dim, num_units):
        super().__init__()
        self.tensor_configs = tensor_configs
        self.lf = tensor_configs['features_positional_encoding_degree']
        self.lv = tensor_configs['views_positional_encoding_degree']
        self.features_dimension = features_dim
        self.use_view_dirs = tensor_configs['use_view_dirs']
        self.input_dim = features_dim * (2 * self.lf + 1) + (3 * (2 * self.lv + 1) if self.use_view_dirs else 0)
        layer1 = torch.nn.Linear(self.input_dim, num_units)
        layer2 = torch.nn.Linear(num_units, num_units)
        layer3 = torch.nn.Linear(num_units, 3)
        self.mlp = torch.nn.Sequential(layer1, torch.nn.ReLU(inplace=True), layer2, torch.nn.ReLU(inplace=True), layer3,
                                       torch.nn.Sigmoid())
        torch.nn.init.constant_(self.mlp[-2].bias, 0)

    def forward(self, input_batch):
        x = T.positional_encoding(input_batch['features'], self.lf)
        if self.tensor_configs['view_dependent_color']:
            x = torch.cat([x, T.positional_encoding(input_batch['view_dirs'], self.lv)], -1)
        h = T.linear(x, self.mlp[0].weight, self.mlp[0].bias, _lib.SRF_ACT_RELU)
        h = T.linear(h, self.mlp[2].weight, self.mlp[2].bias, _lib.SRF_ACT_RELU)
        return {'color': T.linear(h, self.mlp[4].weight, self.mlp[4].bias, _lib.SRF_ACT_SIGMOID)}


class GbVmTensor(torch.nn.Module):
    """LowRankTensor + VmDecomposedTensor (SimpleTensoRF09.py:582-961, 1126-1320)."""

    DECOMPOSITION = 'VectorMatrix'

    def __init__(self, name, configs, tensor_configs, model_configs):
        super().__init__()
        if tensor_configs['decomposition_type'] != self.DECOMPOSITION:
            raise ValueError(f"{type(self).__name__} is the {self.DECOMPOSITION} decomposition, configs ask for "
                             f"{tensor_configs['decomposition_type']} (use make_tensor_model)")
        if tensor_configs.get('predict_visibility', False):
            raise NotImplementedError('predict_visibility is not supported')
        self.name = name
        self.configs = configs
        self.tensor_configs = tensor_configs
        self.model_configs = model_configs
        self.ndc = configs['data_loader']['ndc']
        self.predict_visibility = False
        self.matrix_axes, self.vector_axes = MATRIX_AXES, VECTOR_AXES
        for b, shape, dt in (('bounding_box', (2, 3), None), ('resolution', (3,), None), ('num_samples', (), 'i'),
                             ('bounding_box_size', (3,), None), ('voxel_length', (3,), None), ('step_size', (), None)):
            self.register_buffer(b, torch.zeros(shape) if dt is None else torch.tensor(0))
        bbox = torch.tensor(tensor_configs.get('bounding_box', model_configs['bounding_box']), dtype=torch.float32)
        self.update_tensor_params(compute_resolution_in_voxels(tensor_configs['num_voxels_initial'], bbox), bbox)
        self.alpha_mask = None
        self.optimizers = None
        self.build_tensor()
        self.basis_matrix_color = torch.nn.Linear(sum(tensor_configs['num_components_color']),
                                                  tensor_configs['features_dimension_color'], bias=False)
        self.density_mode = {'ReLU': 0, 'SoftPlus': 1}[tensor_configs['density_predictor']]
        self.density_offset = float(tensor_configs.get('density_offset', 0.0))
        if tensor_configs['color_predictor'] != 'MLP_Features':
            raise NotImplementedError(tensor_configs['color_predictor'])
        self.color_predictor = MlpFeaturesColorPredictor(tensor_configs, tensor_configs['features_dimension_color'],
                                                         tensor_configs['num_units_color_predictor'])
        # configs['model']['precision']: 'fp32' (plain) or 'bf16' / 'fp16' (renderer MLP on the tensor cores)
        self.precision = _precision(configs)
        self._register_load_state_dict_pre_hook(self._load_hook)

    # ------------------------------------------------------------ geometry --
    def update_tensor_params(self, new_resolution, new_bounding_box):
        """SimpleTensoRF09.py:652-665."""
        self.bounding_box = new_bounding_box.float()
        self.bounding_box_size = self.bounding_box[1] - self.bounding_box[0]
        self.resolution = new_resolution.long()
        self.voxel_length = self.bounding_box_size / (self.resolution - 1)
        nvps = self.tensor_configs['num_voxels_per_sample']
        self.step_size = torch.mean(self.voxel_length) * nvps
        n = (torch.linalg.norm(self.resolution.float()) / nvps).round().long()
        self.num_samples = torch.clamp(n, max=int(self.tensor_configs['num_samples_max']))

    def build_tensor(self):
        """VmDecomposedTensor.build_tensor (:1140-1152): density and colour planes + lines."""
        tc = self.tensor_configs
        self.matrices_density, self.vectors_density = self.create_decomposed_tensor(tc['num_components_density'],
                                                                                    self.resolution)
        self.matrices_color, self.vectors_color = self.create_decomposed_tensor(tc['num_components_color'],
                                                                                self.resolution)

    def density_features(self, pts):
        return T.vm_density(self._grid('density'), pts)

    def color_features(self, pts):
        return T.vm_color(self._grid('color'), pts)

    def tensor_parameters(self):
        """The grid parameters in the reference's optimizer order (:1167-1194)."""
        return list(self.vectors_density) + list(self.matrices_density) + list(self.vectors_color) + \
            list(self.matrices_color)

    def create_decomposed_tensor(self, num_components, resolution, scale=0.1):
        """Planes (1,R,res[m1],res[m0]) and lines (1,R,res[v],1), stored channels-last."""
        mats, vecs = [], []
        for i in range(3):
            m0, m1 = MATRIX_AXES[i]
            v = VECTOR_AXES[i]
            mats.append(torch.nn.Parameter(T.to_channels_last(
                scale * torch.randn(1, num_components[i], int(resolution[m1]), int(resolution[m0])))))
            vecs.append(torch.nn.Parameter(T.to_channels_last(
                scale * torch.randn(1, num_components[i], int(resolution[v]), 1))))
        return torch.nn.ParameterList(mats), torch.nn.ParameterList(vecs)

    def _grid(self, kind):
        mats = self.matrices_density if kind == 'density' else self.matrices_color
        vecs = self.vectors_density if kind == 'density' else self.vectors_color
        for p in list(mats) + list(vecs):
            if not p.is_contiguous(memory_format=torch.channels_last):
                p.data = T.to_channels_last(p.data)
        return T.VmGridTensors(list(mats), list(vecs), [int(r) for r in cached_host(self, 'res', self.resolution)])

    def get_trainable_parameters(self, optimizer_configs):
        """SimpleTensoRF09.py:1167-1194."""
        tensor_params = torch.nn.ParameterList()
        network_params = torch.nn.ParameterList()
        tensor_params.extend(self.tensor_parameters())
        network_params.extend(self.basis_matrix_color.parameters())
        network_params.extend(self.color_predictor.parameters())
        return [{'name': f'{self.name}_tensor_params', 'params': tensor_params,
                 'lr': optimizer_configs['lr_initial_tensor']},
                {'name': f'{self.name}_network_params', 'params': network_params,
                 'lr': optimizer_configs['lr_initial_network']}]

    # ------------------------------------------------------------- forward --
    def forward(self, input_dict, retraw):
        """LowRankTensor.forward (SimpleTensoRF09.py:701-761) on the CUDA path.

        Three phases separated by the two host reads of a sample count (valid
        samples, then surface samples), which size the compacted launches;
        :func:`forward_models` runs the phases of several models side by side so
        that one host read serves them all."""
        st = self.forward_begin(input_dict)
        self.forward_density(st, int(st['cnt_v'].item()))
        return self.forward_color(st, int(st['cnt_s'].item()), retraw)

    def forward_begin(self, input_dict):
        """Validity (bounding box and alpha mask, SimpleTensoRF09.py:705-710) and
        the compaction of the valid samples; the count stays on the device."""
        z = input_dict['z_vals_ndc'] if self.ndc else input_dict['z_vals']
        o, d = (input_dict['rays_o_ndc'], input_dict['rays_d_ndc']) if self.ndc else \
            (input_dict['rays_o'], input_dict['rays_d'])
        n, s = z.shape
        rows = n * s
        dev = z.device
        bbox = cached_host(self, 'bbox', self.bounding_box)
        pn = torch.empty(rows, 3, device=dev)
        mask = torch.empty(rows, dtype=torch.uint8, device=dev)
        vol = None
        vd = vh = vw = 0
        abox = None
        if self.alpha_mask is not None:
            vol = self.alpha_mask.volume()
            vd, vh, vw = vol.shape
            abox = _lib.host_floats(cached_host(self.alpha_mask, 'bbox', self.alpha_mask.bounding_box))
        _lib.call('srf_tensorf_sample_mask', F._ptr(o.contiguous()), F._ptr(d.contiguous()), F._ptr(z.contiguous()),
                  n, s, _lib.host_floats(bbox), F._ptr(vol), vd, vh, vw, abox, F._ptr(pn), F._ptr(mask), F._stream())
        idx_v, cnt_v = T.compact(mask)
        return {'input': input_dict, 'z': z, 'n': n, 's': s, 'pn': pn, 'idx_v': idx_v, 'cnt_v': cnt_v}

    def forward_density(self, st, nv, capacity=False):
        """Density on the nv valid samples (uneven per ray: gather, VM lookup,
        activation, SimpleTensoRF09.py:1214-1239), the volume-rendering weights
        (:767-814) and the compaction of the surface samples (weights above the
        threshold, :726); that count stays on the device.

        With ``capacity`` nv is an upper bound chosen without reading the device
        count (graph capture): rows past the count are zero points whose features
        nothing reads, and a count above nv is the caller's to detect."""
        input_dict, z, n, s, pn = st['input'], st['z'], st['n'], st['s'], st['pn']
        rows = n * s
        dev = z.device
        idx_v, cnt_v = st['idx_v'], st['cnt_v']
        pv = T.gather_rows(pn, idx_v, cnt_v, nv, zero_tail=capacity)
        feat = self.density_features(pv) if nv else torch.zeros(0, device=dev)
        sigma = T.density_activation(feat, idx_v, cnt_v, rows, self.density_mode, self.density_offset).view(n, s)
        # the density pass composites no colour (rgb None reads as zeros)
        vr = F.composite(sigma, None, z, input_dict['rays_d'], ndc=self.ndc, rays_o=input_dict['rays_o'],
                         rays_d_ndc=input_dict.get('rays_d_ndc'),
                         distance_scale=self.tensor_configs['distance_scale'])
        out = {k: vr[k] for k in ('acc', 'alpha', 'visibility', 'weights', 'depth', 'depth_var')}
        if self.ndc:
            out['depth_ndc'], out['depth_var_ndc'] = vr['depth_ndc'], vr['depth_var_ndc']
        w = vr['weights']
        smask = torch.empty(rows, dtype=torch.uint8, device=dev)
        _lib.call('srf_threshold_mask', F._ptr(w.detach().contiguous()), rows,
                  float(self.tensor_configs['ray_marching_weight_threshold']), F._ptr(smask), F._stream())
        idx_s, cnt_s = T.compact(smask)
        st.update({'nv': nv, 'sigma': sigma, 'out': out, 'idx_s': idx_s, 'cnt_s': cnt_s})

    def forward_color(self, st, ns, retraw, capacity=False):
        """Colour on the ns surface samples (SimpleTensoRF09.py:1241-1272 and the
        renderer MLP), compositing of the colour and the white background
        (:743-747).  ``capacity``: ns is an upper bound, as in forward_density
        (rows past the count render zero points whose colours nothing reads
        and whose gradients are zero)."""
        input_dict, n, s, pn, out = st['input'], st['n'], st['s'], st['pn'], st['out']
        rows = n * s
        dev = pn.device
        idx_s, cnt_s = st['idx_s'], st['cnt_s']
        w = out['weights']
        self.last_sample_counts = None if capacity else {'marched': rows, 'valid': st['nv'], 'surface': ns}
        if ns:
            ps = T.gather_rows(pn, idx_s, cnt_s, ns, zero_tail=capacity)
            feats = self.color_features(ps)
            view_s = None
            if self.tensor_configs['view_dependent_color']:
                view_s = T.gather_rows(input_dict['view_dirs'].contiguous().float(), idx_s, cnt_s, ns, s,
                                       zero_tail=capacity)
            if self.precision == _lib.SRF_PRECISION_FP32:
                cin = {'features': T.linear(feats, self.basis_matrix_color.weight)}
                if view_s is not None:
                    cin['view_dirs'] = view_s
                rgb_s = self.color_predictor(cin)['color']
            else:
                cp = self.color_predictor
                desc = _lib.RendererDesc(feats.shape[1], cp.features_dimension, cp.mlp[0].out_features, cp.lf, cp.lv,
                                         int(view_s is not None))
                rgb_s = T.renderer_tc(desc, self.precision, feats, view_s,
                                      [self.basis_matrix_color.weight, cp.mlp[0].weight, cp.mlp[0].bias,
                                       cp.mlp[2].weight, cp.mlp[2].bias, cp.mlp[4].weight, cp.mlp[4].bias])
            rgb = T.scatter_rows(rgb_s, idx_s, cnt_s, rows).view(n, s, 3)
        else:
            rgb = torch.zeros(n, s, 3, device=dev)
        rgb_map = T.weighted_sum(w, rgb)
        if self.configs['model']['white_bkgd'] or (self.training and torch.rand((1,)) < 0.5):
            rgb_map = rgb_map + (1 - out['acc'][..., None])
        out['rgb'] = rgb_map
        if retraw:
            out['raw_sigma'] = st['sigma'][..., None]
            out['raw_rgb'] = rgb
        return out

    def host_geometry(self):
        """(bbox as 6 floats, num_samples, step_size) on the host, cached between resizes."""
        return (cached_host(self, 'bbox', self.bounding_box), int(cached_host(self, 'num_samples', self.num_samples)[0]),
                float(cached_host(self, 'step_size', self.step_size)[0]))

    def normalize_points(self, pts):
        """SimpleTensoRF09.py:763-765."""
        return ((pts - self.bounding_box[0]) / self.bounding_box_size) * 2 - 1

    # ------------------------------------------------ training maintenance --
    def run_model_modifications(self, iter_num):
        """SimpleTensoRF09.py:821-830."""
        if self.training and iter_num in self.tensor_configs['alpha_mask_update_iters']:
            bbox_new = self.update_alpha_mask(iter_num)
            if iter_num == self.tensor_configs['alpha_mask_update_iters'][0]:
                self.shrink_tensor(bbox_new)
        if self.training and iter_num in self.tensor_configs['tensor_upsampling_iters']:
            self.upsample_model_resolution(iter_num)
            self.reconfigure_optimizer()

    def get_new_num_voxels(self, iter_num):
        """SimpleTensoRF09.py:838-847: log-linear schedule between initial and final voxel counts."""
        iters = self.tensor_configs['tensor_upsampling_iters']
        k = iters.index(iter_num) + 1
        lo = numpy.log(self.tensor_configs['num_voxels_initial'])
        hi = numpy.log(self.tensor_configs['num_voxels_final'])
        return int(numpy.round(numpy.exp(lo + (hi - lo) * k / len(iters))))

    def upsample_model_resolution(self, iter_num):
        res = compute_resolution_in_voxels(self.get_new_num_voxels(iter_num), self.bounding_box)
        self.update_tensor_params(res, self.bounding_box)
        self.resample_tensor(self.resolution)

    def resample_tensor(self, res):
        self.matrices_density, self.vectors_density = self.resize(self.matrices_density, self.vectors_density, res)
        self.matrices_color, self.vectors_color = self.resize(self.matrices_color, self.vectors_color, res)

    def resize(self, mats, vecs, res):
        """Bilinear (align_corners) resampling of planes and lines to a new resolution
        (:1284-1301) on the srf_resample_grid kernel."""
        new_m, new_v = [], []
        for i in range(3):
            m0, m1 = MATRIX_AXES[i]
            v = VECTOR_AXES[i]
            new_m.append(torch.nn.Parameter(T.resample_grid(T.to_channels_last(mats[i].data), int(res[m1]),
                                                            int(res[m0]))))
            new_v.append(torch.nn.Parameter(T.resample_grid(T.to_channels_last(vecs[i].data), int(res[v]), 1)))
        return torch.nn.ParameterList(new_m), torch.nn.ParameterList(new_v)

    def reshape_tensor(self, res):
        """Planes and lines of the shapes of resolution res (channels-last, on their
        device), values left for a checkpoint to fill (the load hook)."""
        for kind in ('density', 'color'):
            mats = getattr(self, f'matrices_{kind}')
            vecs = getattr(self, f'vectors_{kind}')
            new_m, new_v = [], []
            for i in range(3):
                m0, m1 = MATRIX_AXES[i]
                v = VECTOR_AXES[i]
                r = mats[i].shape[1]
                new_m.append(torch.nn.Parameter(T.to_channels_last(
                    torch.zeros(1, r, int(res[m1]), int(res[m0]), device=mats[i].device))))
                new_v.append(torch.nn.Parameter(T.to_channels_last(
                    torch.zeros(1, vecs[i].shape[1], int(res[v]), 1, device=vecs[i].device))))
            setattr(self, f'matrices_{kind}', torch.nn.ParameterList(new_m))
            setattr(self, f'vectors_{kind}', torch.nn.ParameterList(new_v))

    @torch.no_grad()
    def compute_alpha(self, xyz, length):
        """SimpleTensoRF09.py:878-897: 1 - exp(-sigma * length) on world points."""
        pn = self.normalize_points(xyz).contiguous().float()
        keep = torch.ones(xyz.shape[0], dtype=torch.uint8, device=xyz.device)
        if self.alpha_mask is not None:
            keep = (self.alpha_mask.sample_alpha(xyz) > 0).to(torch.uint8)
        idx, cnt = T.compact(keep)
        nv = int(cnt.item())
        feat = self.density_features(T.gather_rows(pn, idx, cnt, nv)) if nv else torch.zeros(0, device=xyz.device)
        sigma = T.density_activation(feat, idx, cnt, xyz.shape[0], self.density_mode, self.density_offset)
        return 1 - torch.exp(-sigma * length)

    @torch.no_grad()
    def dense_alpha(self):
        """Alpha of the density on every grid node, z-major (res[2], res[1], res[0])
        (:849-858, 878-897), on the srf_vm_alpha_grid kernel."""
        am = self.alpha_mask
        return T.alpha_grid(self._grid('density'), cached_host(self, 'bbox', self.bounding_box),
                            None if am is None else am.volume(),
                            None if am is None else cached_host(am, 'bbox', am.bounding_box),
                            float(cached_host(self, 'step_size', self.step_size)[0]), self.density_mode,
                            self.density_offset)

    @torch.no_grad()
    def update_alpha_mask(self, iter_num):
        """SimpleTensoRF09.py:849-876: dense alpha of the density on the grid's nodes
        (srf_vm_alpha_grid), 3^3 max-pool and threshold with the occupied node range
        (srf_alpha_pool_threshold); returns the occupied box."""
        gs = [int(r) for r in self.resolution]
        alpha = self.dense_alpha()
        vol, rng = T.alpha_pool_threshold(alpha, self.tensor_configs['alpha_mask_threshold'])
        if rng is None:
            raise RuntimeError('update_alpha_mask: no grid node is occupied (the reference fails on the empty box)')
        self.alpha_mask = AlphaGridMask(vol, self.bounding_box)
        # node coordinates as the reference forms them: CPU linspace, then
        # bbox_lo (1 - s) + bbox_hi s (:851-856)
        lo_hi = self.bounding_box.detach().cpu().float()
        box = torch.empty(2, 3)
        for a in range(3):
            s = torch.linspace(0, 1, gs[a])
            idx = torch.tensor([rng[0][a], rng[1][a]])
            box[:, a] = lo_hi[0, a] * (1 - s[idx]) + lo_hi[1, a] * s[idx]
        return box.to(self.bounding_box.device)

    @torch.no_grad()
    def shrink_tensor(self, bbox_new):
        """SimpleTensoRF09.py:899-914, 1303-1320: crop the grid to the occupied box."""
        lo, hi = bbox_new
        t_l = torch.round((lo - self.bounding_box[0]) / self.voxel_length).long()
        b_r = torch.round((hi - self.bounding_box[0]) / self.voxel_length).long() + 1
        b_r = torch.stack([b_r, self.resolution]).amin(0)
        if not torch.equal(self.alpha_mask.resolution, self.resolution):
            tl_r, br_r = t_l / (self.resolution - 1), (b_r - 1) / (self.resolution - 1)
            fixed = torch.zeros_like(bbox_new)
            fixed[0] = (1 - tl_r) * self.bounding_box[0] + tl_r * self.bounding_box[1]
            fixed[1] = (1 - br_r) * self.bounding_box[0] + br_r * self.bounding_box[1]
            bbox_new = fixed
        self.update_tensor_params(b_r - t_l, bbox_new)
        self.crop_tensor(t_l, b_r)

    def crop_tensor(self, t_l, b_r):
        """The slicing of shrink_tensor (:1303-1320) on the srf_crop_grid kernel."""
        t_l, b_r = [int(x) for x in t_l], [int(x) for x in b_r]
        for plist, vlist in ((self.matrices_density, self.vectors_density), (self.matrices_color, self.vectors_color)):
            for i in range(3):
                m0, m1 = MATRIX_AXES[i]
                v = VECTOR_AXES[i]
                vlist[i] = torch.nn.Parameter(T.crop_grid(T.to_channels_last(vlist[i].data), t_l[v], b_r[v], 0, 1))
                plist[i] = torch.nn.Parameter(T.crop_grid(T.to_channels_last(plist[i].data), t_l[m1], b_r[m1],
                                                          t_l[m0], b_r[m0]))

    def reconfigure_optimizer(self):
        """SimpleTensoRF09.py:916-944: replace this model's param groups in the optimizer."""
        opt = self.optimizers['optimizer_nerf']
        cfg = next(c for c in self.configs['optimizers'] if c['name'] == 'optimizer_main')
        groups = self.get_trainable_parameters(cfg)
        names = {g['name'] for g in groups}
        keep = [g for g in opt.param_groups if g.get('name') not in names]
        dropped = [p for g in opt.param_groups if g.get('name') in names for p in g['params']]
        for p in dropped:
            opt.state.pop(p, None)
        opt.param_groups = keep
        for g in groups:
            opt.add_param_group(g)

    def _load_hook(self, sd, prefix, *args, **kwargs):
        """SimpleTensoRF09.py:946-961, 1196-1212: rebuild the alpha mask and resize the grid
        to the checkpoint's resolution before the tensors are copied in."""
        key = f'{prefix}alpha_mask.alpha_volume'
        if key in sd:
            self.alpha_mask = AlphaGridMask(sd[key].float(), sd[f'{prefix}alpha_mask.bounding_box'])
        res = sd.get(f'{prefix}resolution')
        if res is not None:
            self.reshape_tensor(res)


class GbCpTensor(GbVmTensor):
    """LowRankTensor + CpDecomposedTensor (SimpleTensoRF09.py:964-1123): density and colour
    from three lines each (vector_axes (2, 1, 0)), on the CP lookup kernels."""

    DECOMPOSITION = 'CandecompParafac'

    def build_tensor(self):
        """CpDecomposedTensor.build_tensor (:979-987)."""
        tc = self.tensor_configs
        self.vectors_density = self.create_decomposed_tensor(tc['num_components_density'], self.resolution)
        self.vectors_color = self.create_decomposed_tensor(tc['num_components_color'], self.resolution)

    def create_decomposed_tensor(self, num_components, resolution, scale=0.1):
        """Lines (1, R, res[vector_axes[i]], 1), R = num_components[0] (:989-996), channels-last."""
        return torch.nn.ParameterList([torch.nn.Parameter(T.to_channels_last(
            scale * torch.randn(1, num_components[0], int(resolution[VECTOR_AXES[i]]), 1))) for i in range(3)])

    def _lines(self, kind):
        lines = self.vectors_density if kind == 'density' else self.vectors_color
        for p in lines:
            if not p.is_contiguous(memory_format=torch.channels_last):
                p.data = T.to_channels_last(p.data)
        return list(lines)

    def density_features(self, pts):
        return T.cp_density(self._lines('density'), cached_host(self, 'res', self.resolution), pts)

    def color_features(self, pts):
        return T.cp_color(self._lines('color'), cached_host(self, 'res', self.resolution), pts)

    def tensor_parameters(self):
        """(:998-1026): density lines, then colour lines."""
        return list(self.vectors_density) + list(self.vectors_color)

    def resample_tensor(self, res):
        """upsample_vectors (:1106-1116) on the srf_resample_grid kernel."""
        def up(vecs):
            return torch.nn.ParameterList([torch.nn.Parameter(T.resample_grid(
                T.to_channels_last(vecs[i].data), int(res[VECTOR_AXES[i]]), 1)) for i in range(3)])
        self.vectors_density = up(self.vectors_density)
        self.vectors_color = up(self.vectors_color)

    def reshape_tensor(self, res):
        for kind in ('density', 'color'):
            vecs = getattr(self, f'vectors_{kind}')
            setattr(self, f'vectors_{kind}', torch.nn.ParameterList([torch.nn.Parameter(T.to_channels_last(
                torch.zeros(1, vecs[i].shape[1], int(res[VECTOR_AXES[i]]), 1, device=vecs[i].device)))
                for i in range(3)]))

    @torch.no_grad()
    def dense_alpha(self):
        """Alpha on every grid node through the CP density lookups, z-major."""
        gs = [int(r) for r in self.resolution]
        dev = self.bounding_box.device
        t = [torch.linspace(0, 1, g).to(dev) for g in gs]
        samples = torch.stack(torch.meshgrid(*t, indexing='ij'), -1)
        xyz = self.bounding_box[0] * (1 - samples) + self.bounding_box[1] * samples
        alpha = torch.empty(gs, device=dev).view(-1)
        flat = xyz.view(-1, 3)
        chunk = 1 << 22
        for a in range(0, flat.shape[0], chunk):
            alpha[a:a + chunk] = self.compute_alpha(flat[a:a + chunk], self.step_size)
        return alpha.view(gs).clamp(0, 1).transpose(0, 2).contiguous()

    def crop_tensor(self, t_l, b_r):
        """shrink_tensor (:1118-1123) on the srf_crop_grid kernel."""
        t_l, b_r = [int(x) for x in t_l], [int(x) for x in b_r]
        for vlist in (self.vectors_density, self.vectors_color):
            for i in range(3):
                v = VECTOR_AXES[i]
                vlist[i] = torch.nn.Parameter(T.crop_grid(T.to_channels_last(vlist[i].data), t_l[v], b_r[v], 0, 1))


def make_tensor_model(name, configs, tensor_configs, model_configs):
    """SimpleTensoRF.get_tensor_model (SimpleTensoRF09.py:534-544)."""
    kinds = {GbVmTensor.DECOMPOSITION: GbVmTensor, GbCpTensor.DECOMPOSITION: GbCpTensor}
    kind = tensor_configs['decomposition_type']
    if kind not in kinds:
        raise RuntimeError(f'Unknown tensor decomposition: {kind}')
    return kinds[kind](name, configs, tensor_configs, model_configs)


def _host_counts(counts):
    """Device sample counts -> host ints in one device-to-host read."""
    return [int(v) for v in torch.cat([c.reshape(1) for c in counts]).cpu().tolist()]


_SIDE_STREAMS = {}


def _side_stream(device, i):
    key = (str(device), i)
    if key not in _SIDE_STREAMS:
        _SIDE_STREAMS[key] = _lib.new_stream(device)
    return _SIDE_STREAMS[key]


def forward_models(calls, retraw, concurrent=True):
    """``[model(input_dict, retraw) for model, input_dict in calls]`` with the
    phases of every model enqueued before each host read of the sample counts:
    two device-to-host reads for the whole list instead of two per model (the
    GPU holds every model's pending work while the host waits).  With
    ``concurrent`` every model after the first runs on a stream of its own, so
    the models' kernels overlap (their backward passes follow the same streams);
    the outputs are joined to the caller's stream.  Outputs are those of calling
    the models one by one."""
    main = torch.cuda.current_stream()
    streams = [main] * len(calls)
    if concurrent and len(calls) > 1:
        dev = main.device
        streams = [main] + [_side_stream(dev, i) for i in range(1, len(calls))]
        for (_, inp), st in zip(calls[1:], streams[1:]):
            st.wait_stream(main)
            for t in inp.values():
                if torch.is_tensor(t) and t.is_cuda:
                    t.record_stream(st)
    sides = streams[1:] if streams[0] is not streams[-1] else []

    def join():
        for st in sides:
            main.wait_stream(st)

    states = []
    for (m, inp), st in zip(calls, streams):
        with torch.cuda.stream(st):
            states.append(m.forward_begin(inp))
    join()
    for (m, _), st, state, nv in zip(calls, streams, states, _host_counts([x['cnt_v'] for x in states])):
        with torch.cuda.stream(st):
            m.forward_density(state, nv)
    join()
    outs = []
    for (m, _), st, state, ns in zip(calls, streams, states, _host_counts([x['cnt_s'] for x in states])):
        with torch.cuda.stream(st):
            outs.append(m.forward_color(state, ns, retraw))
    join()
    for out, st in zip(outs, streams):
        if st is not main:
            for t in out.values():
                if torch.is_tensor(t) and t.is_cuda:
                    t.record_stream(main)
    return outs


class GbSimpleTensoRF(torch.nn.Module):
    """Drop-in for ``SimpleTensoRF`` (src/models/SimpleTensoRF09.py:16)."""

    def __init__(self, configs, model_configs):
        super().__init__()
        self.configs = configs
        self.model_configs = model_configs
        self.ndc = configs['data_loader']['ndc']
        self.coarse_model_needed = 'coarse_model' in configs['model']
        self.fine_model_needed = 'fine_model' in configs['model']
        self.predict_visibility = False
        self.nerf_synthetic = configs.get('database') == 'NeRF_Synthetic'
        self.coarse_model = self.fine_model = None
        self.augmentations_needed = 'augmentations' in configs['model']
        if self.augmentations_needed:
            self.augmented_models = []
            self.augmented_models_nn = []
        self.build_nerf()
        self.optimizers = None
        self.train_data_preprocessor = None

    def build_nerf(self):
        m = self.configs['model']
        if self.coarse_model_needed:
            self.coarse_model = make_tensor_model('coarse_model', self.configs, m['coarse_model'], self.model_configs)
        if self.fine_model_needed:
            self.fine_model = make_tensor_model('fine_model', self.configs, m['fine_model'], self.model_configs)
        self.intrinsics_learner = IntrinsicsLearner(numpy.array(self.model_configs['intrinsics']),
                                                    learn_focal=m['learn_camera_focal_length'])
        self.extrinsics_learner = ExtrinsicsLearner(numpy.array(self.model_configs['extrinsics']),
                                                    learn_rotation=m['learn_camera_rotation'],
                                                    learn_translation=m['learn_camera_translation'])
        if self.augmentations_needed:
            for aug in m['augmentations']:
                nn_dict = ModuleDict()
                entry = {'name': aug['name'], 'coarse_model': None, 'fine_model': None}
                for key in ('coarse_model', 'fine_model'):
                    if key in aug:
                        entry[key] = make_tensor_model(f"{aug['name']}_{key}", self.configs, aug[key],
                                                       self.model_configs)
                        nn_dict[key] = entry[key]
                self.augmented_models.append(entry)
                self.augmented_models_nn.append(nn_dict)
            self.augmented_models_nn = ModuleList(self.augmented_models_nn)

    def _models(self):
        ms = [self.coarse_model, self.fine_model]
        if self.augmentations_needed:
            for a in self.augmented_models:
                ms += [a['coarse_model'], a['fine_model']]
        return [x for x in ms if x is not None]

    def __setattr__(self, name, value):
        super().__setattr__(name, value)
        if name == 'optimizers' and value is not None:
            for mdl in self._models():
                mdl.optimizers = value

    def get_trainable_parameters(self, optimizer_configs):
        params = []
        for mdl in self._models():
            params.extend(mdl.get_trainable_parameters(optimizer_configs))
        return params

    def rebuild_camera_params_learners(self, *, intrinsics=None, extrinsics=None, device):
        m = self.configs['model']
        if intrinsics is not None:
            self.intrinsics_learner = IntrinsicsLearner(intrinsics, m['learn_camera_focal_length']).to(device)
        if extrinsics is not None:
            self.extrinsics_learner = ExtrinsicsLearner(extrinsics, m['learn_camera_rotation'],
                                                        m['learn_camera_translation']).to(device)

    def forward(self, input_batch, *, retraw=False, sec_views_vis=False, mode=None):
        """SimpleTensoRF09.py:133-162."""
        check_pose_learning(self)
        input_batch = {k: (dict(v) if isinstance(v, dict) else v) for k, v in input_batch.items()}
        if 'common_data' in input_batch:
            for key, val in input_batch['common_data'].items():
                if isinstance(val, torch.Tensor):
                    input_batch['common_data'][key] = val[0]
        if self.training and mode != 'test_camera_params_optimization' and input_batch.get('sub_batch_index') == 0:
            for mdl in self._models():
                mdl.run_model_modifications(input_batch['iter_num'])
        image_id = input_batch['pixel_id'][:, 0]
        intrinsics = self.intrinsics_learner(image_id)
        extrinsics = self.extrinsics_learner(image_id)
        all_ext = self.extrinsics_learner(torch.arange(input_batch['num_frames']).to(image_id))
        input_batch['intrinsics'], input_batch['extrinsics'] = intrinsics, extrinsics
        out = {} if mode == 'camera_params_only' else self.render(input_batch, retraw=retraw or self.training,
                                                                  mode=mode)
        out['intrinsics'], out['extrinsics'], out['extrinsics_all'] = intrinsics, extrinsics, all_ext
        return out

    def render(self, input_dict, *, retraw, mode):
        all_ret = {}
        n = input_dict['pixel_id'].shape[0]
        chunk = self.configs['model']['chunk']
        for i in range(0, n, chunk):
            sub = {k: (v[i:i + chunk] if isinstance(v, (torch.Tensor, numpy.ndarray)) and v.shape[0] == n else v)
                   for k, v in input_dict.items()}
            for k, v in self.render_rays(sub, retraw=retraw, mode=mode).items():
                all_ret.setdefault(k, []).append(v)
        return {k: torch.cat(v, 0) for k, v in all_ret.items()}

    def render_rays(self, input_dict, *, retraw, mode):
        """SimpleTensoRF09.py:194-351."""
        ret = {}
        # mip_nerf_used=True (+0.5 px) and the x-flip of origins/directions (:205-207).
        # The NeRF-Synthetic convention (:205-210) conjugates the pose by
        # diag(1, -1, -1, 1) and keeps the camera-frame y, z signs: that equals the
        # default rays with y and z negated (sign flips, exact), the x-flip undone,
        # and the directions normalised.
        o, d = F.pixel_rays(input_dict['pixel_id'], input_dict['intrinsics'], input_dict['extrinsics'],
                            half_pixel=True)
        flip = torch.tensor([1.0, -1.0, -1.0] if self.nerf_synthetic else [-1.0, 1.0, 1.0], device=o.device)
        o, d = (o * flip).contiguous(), (d * flip).contiguous()
        if self.nerf_synthetic:
            d = (d / torch.linalg.norm(d, dim=1, keepdim=True)).contiguous()
        ret['rays_o'], ret['rays_d'] = o, d
        h, w = self.model_configs['resolution']
        if self.ndc:
            k = input_dict['intrinsics'].float()
            ret['rays_o_ndc'], ret['rays_d_ndc'] = F.ndc_rays(o, d, k[:, 0, 0].contiguous(), k[:, 1, 1].contiguous(),
                                                              h, w, self.model_configs['near'])
        m = self.configs['model']
        if any(m[key]['use_view_dirs'] for key in ('coarse_model', 'fine_model') if key in m):
            if mode == 'static_camera':
                # view directions of the fixed view pose (:222-232): its own rays,
                # without the half pixel and without the x-flip
                n = input_dict['pixel_id'].shape[0]
                cd = input_dict['common_data']
                vi = cd['view_intrinsic']
                vk = (vi[None].repeat(n, 1, 1) if vi is not None else input_dict['intrinsics']).float().contiguous()
                ve = cd['processed_view_pose'][None].repeat(n, 1, 1).float().contiguous()
                vo, vd = F.pixel_rays(input_dict['pixel_id'], vk, ve)
                if self.ndc:
                    _, vd = F.ndc_rays(vo, vd, vk[:, 0, 0].contiguous(), vk[:, 1, 1].contiguous(), h, w,
                                       self.model_configs['near'])
                ret['view_dirs'] = F.view_dirs(vd)
            else:
                ret['view_dirs'] = F.view_dirs(ret['rays_d_ndc'] if self.ndc else d)
        train_augs = self.augmentations_needed and self.training and mode != 'test_camera_params_optimization'

        def model_input(z):
            mi = {'iter_num': input_dict.get('iter_num'), 'z_vals': z, 'rays_o': o, 'rays_d': d}
            if self.ndc:
                mi.update({'z_vals_ndc': z, 'rays_o_ndc': ret['rays_o_ndc'], 'rays_d_ndc': ret['rays_d_ndc']})
            if 'view_dirs' in ret:
                mi['view_dirs'] = ret['view_dirs']
            return mi

        weights_c = z_c = None
        if self.coarse_model_needed:
            z_c = self.get_z_vals_coarse(input_dict, ret, self.coarse_model)
            mi = model_input(z_c)
            # the main and augmented models on the same samples (:244-296), their
            # phases side by side (forward_models)
            augs = [aug for aug in self.augmented_models if aug['coarse_model'] is not None] if train_augs else []
            res = forward_models([(self.coarse_model, mi)] + [(aug['coarse_model'], mi) for aug in augs], retraw)
            outs = res[0]
            weights_c = outs['weights']
            ret['z_vals_coarse'] = z_c
            for k, v in outs.items():
                ret[f'{k}_coarse'] = v
            for aug, aug_out in zip(augs, res[1:]):
                for k, v in aug_out.items():
                    ret[f"{aug['name']}_{k}_coarse"] = v
        if self.fine_model_needed:
            nf = m['fine_model']['num_samples']
            u = torch.rand(z_c.shape[0], nf, device=z_c.device) if (m['perturb'] and self.training) else None
            z_f = F.fine_z(z_c.contiguous(), weights_c.detach(), nf, u)
            mi = model_input(z_f)
            augs = [aug for aug in self.augmented_models if aug['fine_model'] is not None] if train_augs else []
            res = forward_models([(self.fine_model, mi)] + [(aug['fine_model'], mi) for aug in augs], retraw)
            ret['z_vals_fine'] = z_f
            for k, v in res[0].items():
                ret[f'{k}_fine'] = v
            for aug, aug_out in zip(augs, res[1:]):
                for k, v in aug_out.items():
                    ret[f"{aug['name']}_{k}_fine"] = v
        if not retraw:
            for tag, needed in (('coarse', self.coarse_model_needed), ('fine', self.fine_model_needed)):
                if needed:
                    for k in ('z_vals', 'alpha', 'visibility', 'weights'):
                        ret.pop(f'{k}_{tag}', None)
        return ret

    def get_z_vals_coarse(self, input_dict, output_dict, tensor_model):
        """SimpleTensoRF09.py:353-401."""
        n = input_dict['pixel_id'].shape[0]
        bbox, s, step = tensor_model.host_geometry()
        perturb = self.training and self.configs['model']['perturb']
        dev = input_dict['pixel_id'].device
        if self.ndc:
            near, far = self.model_configs['near_ndc'], self.model_configs['far_ndc']
            u = torch.rand(n, s, device=dev) if perturb else None
            return F.stratified_z(n, s, near, far, u, lindisp=self.configs['model']['lindisp'], device=dev)
        near, far = self.model_configs['near'], self.model_configs['far']
        u = torch.rand(n, device=dev) if perturb else None
        return F.aabb_z(output_dict['rays_o'], output_dict['rays_d'], s, bbox, near, far, step, u)


# ModelFactory02 convention (class name = module name minus the two-digit suffix).
SimpleTensoRF = GbSimpleTensoRF
