"""TensoRF VM operators over the srf_gb300 C ABI (SimpleTensoRF09.py:1126-1421).

VM planes/lines keep the reference's logical shapes ``(1, R, H, W)`` /
``(1, R, L, 1)`` but live in ``torch.channels_last`` memory, i.e. physically
``(H, W, R)`` / ``(L, R)``: one bilinear corner is R contiguous floats.  The
TV loss, upsampling, shrinking and Adam of the reference keep working on the
logical view.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from . import functional as F
from ._lib import call
from .functional import _ptr, _require, _stream


def to_channels_last(t):
    """(1,R,H,W) tensor in the physical (H,W,R) layout the VM kernels read."""
    return t.contiguous(memory_format=torch.channels_last)


_DETERMINISTIC_SCATTER = False


def set_deterministic_scatter(on=True):
    """Route the VM grid adjoints (vm_density / vm_color backward) through the
    fixed-point scatter-add (srf_vm_*_backward_fixed), whose gradients are bitwise
    reproducible, instead of the faster FP32 atomics.  Also on whenever
    torch.use_deterministic_algorithms(True) is in effect."""
    global _DETERMINISTIC_SCATTER
    _DETERMINISTIC_SCATTER = bool(on)


def deterministic_scatter():
    return _DETERMINISTIC_SCATTER or torch.are_deterministic_algorithms_enabled()


def zeros_like_all(tensors):
    """Zero tensors shaped, strided (channels-last included) and typed like
    ``tensors``, carved from one zero-filled buffer: one fill launch instead of one
    per tensor.  Each view starts on a 16-byte boundary."""
    if not tensors:
        return []
    spans = []
    total = 0
    for t in tensors:
        n = t.numel()
        spans.append(total)
        total += (n + 3) // 4 * 4
    flat = torch.zeros(max(total, 1), dtype=tensors[0].dtype, device=tensors[0].device)
    return [flat.as_strided(t.shape, t.stride(), off) for t, off in zip(tensors, spans)]


def _is_cl(t):
    return t.dim() == 4 and t.is_contiguous(memory_format=torch.channels_last)


class VmGridTensors:
    """Three plane/line pairs (one VM tensor), as torch tensors."""

    def __init__(self, planes, lines, res):
        self.planes = list(planes)
        self.lines = list(lines)
        self.res = [int(r) for r in res]

    @classmethod
    def from_numpy(cls, planes, lines, res, device):
        pl = [to_channels_last(torch.from_numpy(np.ascontiguousarray(p)).to(device)[None]) for p in planes]
        ln = [to_channels_last(torch.from_numpy(np.ascontiguousarray(l)).to(device)[None]) for l in lines]
        return cls(pl, ln, res)

    def requires_grad_(self, flag=True):
        for x in self.planes + self.lines:
            x.requires_grad_(flag)
        return self

    def tensors(self):
        return self.planes + self.lines

    def plane_grad_numpy(self, i):
        return self.planes[i].grad[0].detach().cpu().numpy()

    def line_grad_numpy(self, i):
        return self.lines[i].grad[0].detach().cpu().numpy()


def _grid_struct(res, planes, lines):
    g = _lib.VmGrid()
    for i in range(3):
        g.res[i] = res[i]
        g.n_comp[i] = planes[i].shape[1]
        if not (_is_cl(planes[i]) and _is_cl(lines[i])):
            raise RuntimeError('VM planes/lines must be channels_last (see to_channels_last)')
        if planes[i].dtype != torch.float32 or not planes[i].is_cuda:
            raise RuntimeError('VM planes/lines must be float32 CUDA tensors')
        g.planes[i] = planes[i].data_ptr()
        g.lines[i] = lines[i].data_ptr()
    return g


class _VmFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, kind, res, pts, *tensors):
        planes, lines = list(tensors[:3]), list(tensors[3:])
        g = _grid_struct(res, planes, lines)
        p = pts.shape[0]
        _require(pts, 'pts', (p, 3))
        if kind == 'density':
            out = torch.empty(p, device=pts.device)
            call('srf_vm_density_forward', ctypes.byref(g), _ptr(pts), p, _ptr(out), _stream())
        else:
            out = torch.empty(p, sum(x.shape[1] for x in planes), device=pts.device)
            call('srf_vm_color_forward', ctypes.byref(g), _ptr(pts), p, _ptr(out), _stream())
        ctx.kind, ctx.res = kind, res
        ctx.save_for_backward(pts, *tensors)
        return out

    @staticmethod
    def backward(ctx, dout):
        pts, *tensors = ctx.saved_tensors
        planes, lines = tensors[:3], tensors[3:]
        grads = zeros_like_all(tensors)
        g = _grid_struct(ctx.res, planes, lines)
        gg = _grid_struct(ctx.res, grads[:3], grads[3:])
        dout = dout.contiguous()
        name = 'srf_vm_density_backward' if ctx.kind == 'density' else 'srf_vm_color_backward'
        if deterministic_scatter():
            nbytes = int(_lib.load().srf_vm_backward_fixed_workspace_size(ctypes.byref(g)))
            ws = torch.empty(nbytes, dtype=torch.uint8, device=pts.device)
            call(name + '_fixed', ctypes.byref(gg), ctypes.byref(g), _ptr(pts), pts.shape[0], _ptr(dout), _ptr(ws),
                 nbytes, _stream())
        else:
            call(name, ctypes.byref(gg), ctypes.byref(g), _ptr(pts), pts.shape[0], _ptr(dout), _stream())
        return (None, None, None) + tuple(grads)


def vm_density(grid, pts):
    """Density features sum_i sum_r plane_i[r] * line_i[r] (SimpleTensoRF09.py:1224-1236)."""
    return _VmFunction.apply('density', grid.res, pts.contiguous(), *grid.tensors())


def vm_color(grid, pts):
    """Colour features (P, sum R_i) = concat_i plane_i * line_i (SimpleTensoRF09.py:1252-1262)."""
    return _VmFunction.apply('color', grid.res, pts.contiguous(), *grid.tensors())


def _cp_struct(res, lines):
    g = _lib.VmGrid()
    for i in range(3):
        g.res[i] = res[i]
        g.n_comp[i] = lines[i].shape[1]
        if not _is_cl(lines[i]) or lines[i].dtype != torch.float32 or not lines[i].is_cuda:
            raise RuntimeError('CP lines must be channels_last float32 CUDA tensors')
        g.lines[i] = lines[i].data_ptr()
    return g


class _CpFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, kind, res, pts, *lines):
        g = _cp_struct(res, lines)
        p = pts.shape[0]
        _require(pts, 'pts', (p, 3))
        if kind == 'density':
            out = torch.empty(p, device=pts.device)
            call('srf_cp_density_forward', ctypes.byref(g), _ptr(pts), p, _ptr(out), _stream())
        else:
            out = torch.empty(p, lines[0].shape[1], device=pts.device)
            call('srf_cp_color_forward', ctypes.byref(g), _ptr(pts), p, _ptr(out), _stream())
        ctx.kind, ctx.res = kind, res
        ctx.save_for_backward(pts, *lines)
        return out

    @staticmethod
    def backward(ctx, dout):
        pts, *lines = ctx.saved_tensors
        grads = zeros_like_all(lines)
        g, gg = _cp_struct(ctx.res, lines), _cp_struct(ctx.res, grads)
        name = 'srf_cp_density_backward' if ctx.kind == 'density' else 'srf_cp_color_backward'
        call(name, ctypes.byref(gg), ctypes.byref(g), _ptr(pts), pts.shape[0], _ptr(dout.contiguous()), _stream())
        return (None, None, None) + tuple(grads)


def cp_density(lines, res, pts):
    """CP density features sum_r prod_i line_i[r] (SimpleTensoRF09.py:1070-1080)."""
    return _CpFunction.apply('density', [int(r) for r in res], pts.contiguous(), *lines)


def cp_color(lines, res, pts):
    """CP colour features (P, R) = prod_i line_i[r] (SimpleTensoRF09.py:1091-1098)."""
    return _CpFunction.apply('color', [int(r) for r in res], pts.contiguous(), *lines)


def alpha_mask_query(volume, pts_norm):
    """AlphaGridMask.sample_alpha(...) > 0 on normalised points (SimpleTensoRF09.py:1342-1349)."""
    vol = volume.reshape(volume.shape[-3:]).contiguous()
    _require(vol, 'alpha_volume')
    p = pts_norm.shape[0]
    _require(pts_norm, 'pts_norm', (p, 3))
    out = torch.empty(p, dtype=torch.uint8, device=pts_norm.device)
    d, h, w = vol.shape
    call('srf_alpha_mask_query', _ptr(vol), d, h, w, _ptr(pts_norm), p, _ptr(out), _stream())
    return out


def compact(mask):
    """Ascending indices of nonzero mask entries; returns (idx (n,), count (1,) device int32)."""
    mask = mask.reshape(-1).contiguous()
    _require(mask, 'mask', dtype=torch.uint8)
    n = mask.numel()
    idx = torch.empty(max(n, 1), dtype=torch.int32, device=mask.device)
    cnt = torch.empty(1, dtype=torch.int32, device=mask.device)
    lib = _lib.load()
    ws = torch.empty(max(lib.srf_compact_workspace_size(n), 4), dtype=torch.uint8, device=mask.device)
    call('srf_compact', _ptr(mask), n, _ptr(idx), _ptr(cnt), _ptr(ws), ws.numel(), _stream())
    return idx, cnt


class _LinearFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, w, b, act, rows_dev):
        rows, k = x.shape
        nn_ = w.shape[0]
        _require(x, 'x')
        _require(w, 'weight', (nn_, k))
        if b is not None:
            _require(b, 'bias', (nn_,))
        y = torch.empty(rows, nn_, device=x.device)
        call('srf_linear_forward', _ptr(y), nn_, _ptr(x), k, _ptr(w), _ptr(b), rows, _ptr(rows_dev), nn_, k, act,
             _stream())
        ctx.act = act
        ctx.has_b = b is not None
        ctx.save_for_backward(x, w, y, rows_dev)
        return y

    @staticmethod
    def backward(ctx, gy):
        x, w, y, rows_dev = ctx.saved_tensors
        rows, k = x.shape
        nn_ = w.shape[0]
        gy = gy.contiguous()
        dx = torch.empty_like(x) if ctx.needs_input_grad[0] else None
        dw = torch.empty_like(w) if ctx.needs_input_grad[1] else None
        db = torch.empty(nn_, device=x.device) if (ctx.has_b and ctx.needs_input_grad[2]) else None
        dz = torch.empty_like(y)
        if dx is not None and rows_dev is not None:
            dx.zero_()
        call('srf_linear_backward', _ptr(dx), k, _ptr(dw), _ptr(db), _ptr(gy), nn_, _ptr(y), nn_, _ptr(x), k, _ptr(w),
             _ptr(dz), rows, _ptr(rows_dev), nn_, k, ctx.act, 0, _stream())
        return dx, dw, db, None, None


class _WeightedSum(torch.autograd.Function):
    """volume_render (SimpleTensoRF09.py:816-819): sum_s w * x."""

    @staticmethod
    def forward(ctx, w, x):
        n, s = w.shape
        c = x.shape[-1]
        out = torch.empty(n, c, device=w.device)
        call('srf_weighted_sum', _ptr(w), _ptr(x), n, s, c, _ptr(out), _stream())
        ctx.save_for_backward(w, x)
        return out

    @staticmethod
    def backward(ctx, g):
        w, x = ctx.saved_tensors
        n, s = w.shape
        dw = torch.empty_like(w) if ctx.needs_input_grad[0] else None
        dx = torch.empty_like(x) if ctx.needs_input_grad[1] else None
        call('srf_weighted_sum_backward', _ptr(w), _ptr(x), _ptr(g.contiguous()), n, s, x.shape[-1], _ptr(dw),
             _ptr(dx), _stream())
        return dw, dx


def weighted_sum(w, x):
    return _WeightedSum.apply(w.contiguous(), x.contiguous())


def gather_rows(src, idx, count, n, row_div=1, zero_tail=False):
    """dst[i] = src[idx[i] // row_div] for i < count (no gradient).  Rows from
    count to n are left unwritten, or zero with ``zero_tail`` (n is then a
    capacity that may exceed the device count)."""
    cols = src.shape[-1]
    dst = (torch.zeros if zero_tail else torch.empty)(n, cols, device=src.device)
    if n:
        call('srf_gather_rows', _ptr(dst), _ptr(src.contiguous()), src.shape[0], _ptr(idx), _ptr(count), n, cols,
             int(row_div), _stream())
    return dst


class _ScatterRows(torch.autograd.Function):
    """Dense (rows, C) zeros with src rows placed at idx (the reference's
    ``rgb[mask] = surface_rgb``, SimpleTensoRF09.py:1247,1271)."""

    @staticmethod
    def forward(ctx, src, idx, count, rows):
        n, c = src.shape
        out = torch.zeros(rows, c, device=src.device)
        if n:
            call('srf_scatter_rows', _ptr(out), rows, _ptr(src.contiguous()), _ptr(idx), _ptr(count), n, c, _stream())
        ctx.save_for_backward(idx, count)
        ctx.n = n
        return out

    @staticmethod
    def backward(ctx, g):
        idx, count = ctx.saved_tensors
        # rows past the device count (a capacity-sized source) get zero gradient
        return gather_rows(g.contiguous(), idx, count, ctx.n, zero_tail=True), None, None, None


def scatter_rows(src, idx, count, rows):
    return _ScatterRows.apply(src, idx, count, rows)


class _DensityActivation(torch.autograd.Function):
    """sigma (rows,) zeros with density_predictor(features) at idx
    (SimpleTensoRF09.py:671-679, 1237-1238)."""

    @staticmethod
    def forward(ctx, feat, idx, count, rows, mode, offset):
        sigma = torch.zeros(rows, device=feat.device)
        n = feat.shape[0]
        if n:
            call('srf_density_activation', _ptr(sigma), rows, _ptr(feat), _ptr(idx), _ptr(count), n, mode,
                 float(offset), _stream())
        ctx.save_for_backward(feat, idx, count)
        ctx.mode, ctx.offset = mode, offset
        return sigma

    @staticmethod
    def backward(ctx, g):
        feat, idx, count = ctx.saved_tensors
        df = torch.zeros_like(feat)
        if feat.shape[0]:
            call('srf_density_activation_backward', _ptr(df), _ptr(g.contiguous()), g.shape[0], _ptr(feat), _ptr(idx),
                 _ptr(count), feat.shape[0], ctx.mode, float(ctx.offset), _stream())
        return df, None, None, None, None, None


def density_activation(feat, idx, count, rows, mode, offset):
    return _DensityActivation.apply(feat.contiguous(), idx, count, rows, mode, offset)


class _PosEnc(torch.autograd.Function):
    """PositionalEncoder.encode (SimpleTensoRF09.py:547-579) with its adjoint."""

    @staticmethod
    def forward(ctx, x, degree):
        m, dims = x.shape
        out = torch.empty(m, dims * (2 * degree + 1), device=x.device)
        if m:
            call('srf_positional_encoding', _ptr(out), out.shape[1], _ptr(x), m, dims, degree, _stream())
        ctx.save_for_backward(x)
        ctx.degree = degree
        return out

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        m, dims = x.shape
        dx = torch.empty_like(x)
        if m:
            g = g.contiguous()
            call('srf_positional_encoding_backward', _ptr(dx), _ptr(x), _ptr(g), g.shape[1], m, None, dims, ctx.degree,
                 _stream())
        return dx, None


def positional_encoding(x, degree):
    return _PosEnc.apply(x.contiguous(), int(degree))


def linear(x, weight, bias=None, act=_lib.SRF_ACT_NONE, rows_dev=None):
    """act(x @ weight.T + bias) on the first ``*rows_dev`` rows (all rows when None)."""
    return _LinearFunction.apply(x.contiguous(), weight.contiguous(), None if bias is None else bias.contiguous(), act,
                                 rows_dev)


class _RendererTcFunction(torch.autograd.Function):
    """basis_matrix_color + MlpFeaturesColorPredictor on the tensor cores
    (srf_tensorf_renderer_*): feats (m, C) and per-sample view dirs (m, 3) -> rgb (m, 3).
    FP16 backwards fit a per-call loss scale to the incoming gradient."""

    @staticmethod
    def forward(ctx, desc, precision, feats, view, *params):
        m = feats.shape[0]
        feats = feats.contiguous()
        params = [p.detach().contiguous() for p in params]
        need_grad = any(ctx.needs_input_grad[2:3]) or any(ctx.needs_input_grad[4:])
        lib = _lib.load()
        ws = torch.empty(max(int(lib.srf_tensorf_renderer_workspace_size(ctypes.byref(desc), m, precision,
                                                                          int(need_grad))), 1),
                         dtype=torch.uint8, device=feats.device)
        if ws.numel() <= 1 and m > 0:
            raise RuntimeError('TensoRF renderer configuration not supported on the tensor-core path '
                               '(units must be 128 or 256)')
        rgb = torch.empty(m, 3, device=feats.device)
        scaler = F.loss_scaler(feats.device) if precision == _lib.SRF_PRECISION_FP16 else None
        _lib.call('srf_tensorf_renderer_forward', ctypes.byref(desc), F._ptr_array(params), F._ptr(feats),
                  F._ptr(view), m, F._ptr(rgb), precision, int(need_grad), F._ptr(ws), ws.numel(), F._ptr(scaler),
                  F._stream())
        ctx.desc, ctx.precision, ctx.m, ctx.scaler = desc, precision, m, scaler
        ctx.ws = ws if need_grad else None
        ctx.params = params
        ctx.save_for_backward(feats)
        return rgb

    @staticmethod
    def backward(ctx, drgb):
        (feats,) = ctx.saved_tensors
        drgb = drgb.contiguous()
        grads = zeros_like_all(ctx.params)
        d_feats = torch.empty_like(feats)
        if ctx.scaler is not None:
            _lib.call('srf_loss_scaler_fit', F._ptr(ctx.scaler), F._ptr(drgb), drgb.numel(), None, 0, 1024.0,
                      F._stream())
        _lib.call('srf_tensorf_renderer_backward', ctypes.byref(ctx.desc), F._ptr_array(ctx.params), F._ptr(feats),
                  F._ptr(drgb), ctx.m, F._ptr_array(grads), F._ptr(d_feats), ctx.precision, F._ptr(ctx.ws),
                  ctx.ws.numel(), F._ptr(ctx.scaler), F._stream())
        ctx.ws = None
        return (None, None, d_feats, None) + tuple(grads)


def renderer_tc(desc, precision, feats, view, params):
    return _RendererTcFunction.apply(desc, precision, feats, view, *params)


# ------------------------------------------------------------ grid maintenance --

def _cl_dims(t):
    """(h, w, comps) of a channels-last (1, comps, h, w) plane or (1, comps, l, 1) line."""
    if not _is_cl(t) or t.dtype != torch.float32 or not t.is_cuda:
        raise RuntimeError('grid tensors must be channels_last float32 CUDA tensors')
    return int(t.shape[2]), int(t.shape[3]), int(t.shape[1])


def resample_grid(t, h_new, w_new):
    """Bilinear align_corners resampling of a plane (1,R,H,W) or line (1,R,L,1) to
    (1,R,h_new,w_new), channels-last (upsample_vectors_and_matrices,
    SimpleTensoRF09.py:1284-1301)."""
    h, w, r = _cl_dims(t)
    out = torch.empty(1, r, h_new, w_new, device=t.device).contiguous(memory_format=torch.channels_last)
    _lib.call('srf_resample_grid', t.data_ptr(), h, w, r, out.data_ptr(), h_new, w_new, _stream(t))
    return out


def crop_grid(t, row0, row1, col0, col1):
    """Rows [row0, row1) x columns [col0, col1) of a plane or line, channels-last
    (shrink_tensor, SimpleTensoRF09.py:1303-1320)."""
    h, w, r = _cl_dims(t)
    out = torch.empty(1, r, row1 - row0, col1 - col0, device=t.device).contiguous(memory_format=torch.channels_last)
    _lib.call('srf_crop_grid', t.data_ptr(), h, w, r, row0, col0, out.data_ptr(), row1 - row0, col1 - col0,
              _stream(t))
    return out


def alpha_grid(grid, bbox, alpha_volume, alpha_bbox, step, density_mode, density_offset):
    """Dense alpha (res[2], res[1], res[0]) on the grid's nodes (update_alpha_mask's
    dense pass with compute_alpha, SimpleTensoRF09.py:849-858, 878-897)."""
    res = grid.res
    dev = grid.planes[0].device
    out = torch.empty(res[2], res[1], res[0], device=dev)
    vd = vh = vw = 0
    vol = None
    if alpha_volume is not None:
        vol = alpha_volume.contiguous().float()
        vd, vh, vw = vol.shape
    g = _grid_struct(res, grid.planes, grid.lines)
    _lib.call('srf_vm_alpha_grid', ctypes.byref(g), _lib.host_floats(bbox), None if vol is None else vol.data_ptr(),
              vd, vh, vw, None if alpha_bbox is None else _lib.host_floats(alpha_bbox), float(step),
              int(density_mode), float(density_offset), out.data_ptr(), _stream(out))
    return out


def alpha_pool_threshold(alpha, threshold):
    """3^3 max-pool and threshold of alpha (gz, gy, gx) -> 0/1 volume, and the
    occupied node range per axis as ((min x, min y, min z), (max x, max y, max z))
    or None when no node is occupied (SimpleTensoRF09.py:859-874)."""
    gz, gy, gx = alpha.shape
    vol = torch.empty_like(alpha)
    bounds = torch.empty(6, dtype=torch.int32, device=alpha.device)
    _lib.call('srf_alpha_pool_threshold', alpha.data_ptr(), gx, gy, gz, float(threshold), vol.data_ptr(),
              bounds.data_ptr(), _stream(alpha))
    b = bounds.cpu().tolist()
    if b[3] < 0:
        return vol, None
    return vol, ((gx - 1 - b[0], gy - 1 - b[1], gz - 1 - b[2]), (b[3], b[4], b[5]))
