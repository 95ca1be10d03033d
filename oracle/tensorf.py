"""Numpy restatement of the Simple-TensoRF (VM) rendering path -- TEST INFRASTRUCTURE ONLY.

Follows ``src/models/SimpleTensoRF09.py`` (paths relative to the reference root).
``grid_sample`` semantics (bilinear / trilinear, ``align_corners=True``, zero
padding) are restated from PyTorch's published CPU kernels, which the reference
calls at SimpleTensoRF09.py:1232-1235, 1258-1261 and 1344.
"""
import numpy as np

from .nerf import composite_forward, composite_backward, positional_encoding, relu, sigmoid, _cumprod  # noqa: F401

MATRIX_AXES = [[0, 1], [0, 2], [1, 2]]   # SimpleTensoRF09.py:1131
VECTOR_AXES = [2, 1, 0]                  # SimpleTensoRF09.py:1132


def _bilinear_taps(gx, gy, h, w):
    """Corner indices and weights of torch's vectorised CPU bilinear sampler
    (align_corners=True): ix = (x + 1) * ((W - 1) / 2), weights from the
    fractional parts (nw = s*e, ne = s*w, sw = n*e, se = n*w)."""
    dt = gx.dtype.type
    ix = (gx + dt(1)) * dt((w - 1) / 2)
    iy = (gy + dt(1)) * dt((h - 1) / 2)
    x0 = np.floor(ix)
    y0 = np.floor(iy)
    fw = ix - x0
    fe = dt(1) - fw
    fn = iy - y0
    fs = dt(1) - fn
    x0 = x0.astype(np.int64)
    y0 = y0.astype(np.int64)
    taps = []
    for dx, dy, wt in ((0, 0, fs * fe), (1, 0, fs * fw), (0, 1, fn * fe), (1, 1, fn * fw)):
        xi, yi = x0 + dx, y0 + dy
        ok = (xi >= 0) & (xi < w) & (yi >= 0) & (yi < h)
        taps.append((np.where(ok, yi, 0), np.where(ok, xi, 0), np.where(ok, wt, dt(0))))
    return taps


def grid_sample_2d(img, gx, gy):
    """img (C,H,W); normalised coords gx (P,) along W, gy (P,) along H -> (C,P)."""
    c, h, w = img.shape
    out = np.zeros((c, gx.shape[0]), dtype=img.dtype)
    for yi, xi, wt in _bilinear_taps(gx, gy, h, w):
        out = out + img[:, yi, xi] * wt[None, :]
    return out


def grid_sample_2d_backward(shape, gx, gy, grad, dtype):
    """Adjoint of :func:`grid_sample_2d` w.r.t. the image (coords are detached, :1225)."""
    c, h, w = shape
    gimg = np.zeros((c, h * w), dtype=np.float64)
    for yi, xi, wt in _bilinear_taps(gx, gy, h, w):
        flat = yi * w + xi
        for ch in range(c):
            # a float64 histogram of the tap contributions (np.add.at semantics, faster)
            gimg[ch] += np.bincount(flat, weights=(grad[ch] * wt).astype(np.float64), minlength=h * w)
    return gimg.reshape(c, h, w).astype(dtype)


def grid_sample_3d_positive(vol, p):
    """AlphaGridMask.sample_alpha (SimpleTensoRF09.py:1342-1349) followed by ``> 0`` (:709).

    vol (D,H,W) of 0/1; p (P,3) normalised (x->W, y->H, z->D).  torch's CPU 3-D
    sampler sums w*v over in-bound corners; with v in {0,1} and w >= 0 the sum is
    positive iff an occupied in-bound corner has a positive weight.
    """
    d, h, w = vol.shape
    dt = p.dtype.type
    ix = ((p[:, 0] + dt(1)) / dt(2)) * dt(w - 1)
    iy = ((p[:, 1] + dt(1)) / dt(2)) * dt(h - 1)
    iz = ((p[:, 2] + dt(1)) / dt(2)) * dt(d - 1)
    x0, y0, z0 = np.floor(ix), np.floor(iy), np.floor(iz)
    x1, y1, z1 = x0 + 1, y0 + 1, z0 + 1
    acc = np.zeros(p.shape[0], dtype=p.dtype)
    corners = [
        (x0, y0, z0, (x1 - ix) * (y1 - iy) * (z1 - iz)),
        (x1, y0, z0, (ix - x0) * (y1 - iy) * (z1 - iz)),
        (x0, y1, z0, (x1 - ix) * (iy - y0) * (z1 - iz)),
        (x1, y1, z0, (ix - x0) * (iy - y0) * (z1 - iz)),
        (x0, y0, z1, (x1 - ix) * (y1 - iy) * (iz - z0)),
        (x1, y0, z1, (ix - x0) * (y1 - iy) * (iz - z0)),
        (x0, y1, z1, (x1 - ix) * (iy - y0) * (iz - z0)),
        (x1, y1, z1, (ix - x0) * (iy - y0) * (iz - z0)),
    ]
    for cx, cy, cz, wt in corners:
        cx, cy, cz = cx.astype(np.int64), cy.astype(np.int64), cz.astype(np.int64)
        ok = (cx >= 0) & (cx < w) & (cy >= 0) & (cy < h) & (cz >= 0) & (cz < d)
        v = vol[np.where(ok, cz, 0), np.where(ok, cy, 0), np.where(ok, cx, 0)]
        acc = acc + np.where(ok, v * wt, dt(0))
    return acc > 0


def aabb_z(rays_o, rays_d, bbox, near, far, step_size, n_samples, u=None):
    """SimpleTensoRF09.py:388-400: AABB entry t_min clamped to [near, far], then
    ``t_min + step * (arange(S) + u_ray)`` with one uniform per ray."""
    dt = rays_o.dtype.type
    vec = np.where(rays_d == 0, dt(1e-6), rays_d)
    ra = (bbox[1] - rays_o) / vec
    rb = (bbox[0] - rays_o) / vec
    t_min = np.clip(np.max(np.minimum(ra, rb), -1), dt(near), dt(far))
    rng = np.arange(n_samples, dtype=rays_o.dtype)[None, :]
    if u is not None:
        rng = rng + u.reshape(-1, 1).astype(rays_o.dtype)
    return t_min[:, None] + dt(step_size) * rng


def normalize_points(pts, bbox):
    """SimpleTensoRF09.py:763-765."""
    dt = pts.dtype.type
    return ((pts - bbox[0]) / (bbox[1] - bbox[0])) * dt(2) - dt(1)


def vm_features(planes, lines, pn):
    """Per-plane products plane_i[r](x_m0, x_m1) * line_i[r](x_v) -> list of (R_i, P)."""
    feats = []
    for i in range(3):
        m0, m1 = MATRIX_AXES[i]
        v = VECTOR_AXES[i]
        pc = grid_sample_2d(planes[i], pn[:, m0], pn[:, m1])
        lc = grid_sample_2d(lines[i], np.zeros_like(pn[:, v]), pn[:, v])
        feats.append((pc, lc))
    return feats


def vm_density(planes, lines, pn):
    """VmDecomposedTensor.get_volume_density (SimpleTensoRF09.py:1214-1239) before the predictor."""
    acc = np.zeros(pn.shape[0], dtype=pn.dtype)
    for pc, lc in vm_features(planes, lines, pn):
        acc = acc + np.sum(pc * lc, 0)
    return acc


def cp_lines(lines, pn):
    """Line i of a CP decomposition at coordinate pn[:, VECTOR_AXES[i]] -> list of (R, P)
    (CpDecomposedTensor.get_volume_density / get_color lookups, SimpleTensoRF09.py:1070-1078)."""
    return [grid_sample_2d(lines[i], np.zeros_like(pn[:, VECTOR_AXES[i]]), pn[:, VECTOR_AXES[i]]) for i in range(3)]


def cp_density(lines, pn):
    """sum_r line_0[r] line_1[r] line_2[r] (SimpleTensoRF09.py:1075-1079) before the predictor."""
    l0, l1, l2 = cp_lines(lines, pn)
    return np.sum(l0 * l1 * l2, 0)


class RendererSpec:
    """MlpFeaturesColorPredictor (SimpleTensoRF09.py:1370-1394)."""

    def __init__(self, features_dim=27, features_pe=2, views_pe=2, units=128, use_view_dirs=True):
        self.F, self.Lf, self.Lv, self.U = features_dim, features_pe, views_pe, units
        self.use_view_dirs = use_view_dirs
        self.in_dim = features_dim * (2 * features_pe + 1) + (3 * (2 * views_pe + 1) if use_view_dirs else 0)

    def param_shapes(self, n_color_components):
        return {
            'basis_matrix_color.weight': (self.F, n_color_components),
            'color_predictor.mlp.0.weight': (self.U, self.in_dim), 'color_predictor.mlp.0.bias': (self.U,),
            'color_predictor.mlp.2.weight': (self.U, self.U), 'color_predictor.mlp.2.bias': (self.U,),
            'color_predictor.mlp.4.weight': (3, self.U), 'color_predictor.mlp.4.bias': (3,),
        }


def renderer_forward(p, spec, feats144, vdirs):
    """basis (SimpleTensoRF09.py:1263) then MlpFeaturesColorPredictor.forward (:1411-1421)."""
    f = feats144 @ p['basis_matrix_color.weight'].T
    x = positional_encoding(f, spec.Lf)
    if spec.use_view_dirs:
        x = np.concatenate([x, positional_encoding(vdirs, spec.Lv)], -1)
    z0 = x @ p['color_predictor.mlp.0.weight'].T + p['color_predictor.mlp.0.bias']
    h0 = relu(z0)
    z1 = h0 @ p['color_predictor.mlp.2.weight'].T + p['color_predictor.mlp.2.bias']
    h1 = relu(z1)
    z2 = h1 @ p['color_predictor.mlp.4.weight'].T + p['color_predictor.mlp.4.bias']
    rgb = sigmoid(z2)
    return rgb, dict(f144=feats144, f=f, x=x, z0=z0, h0=h0, z1=z1, h1=h1, rgb=rgb, vd=vdirs)


def renderer_backward(p, spec, c, drgb):
    """Adjoint of :func:`renderer_forward`; returns (param grads, d feats144)."""
    g = {}
    dt = drgb.dtype.type
    dz2 = drgb * c['rgb'] * (dt(1) - c['rgb'])
    g['color_predictor.mlp.4.weight'] = dz2.T @ c['h1']
    g['color_predictor.mlp.4.bias'] = dz2.sum(0)
    dz1 = (dz2 @ p['color_predictor.mlp.4.weight']) * (c['z1'] > 0)
    g['color_predictor.mlp.2.weight'] = dz1.T @ c['h0']
    g['color_predictor.mlp.2.bias'] = dz1.sum(0)
    dz0 = (dz1 @ p['color_predictor.mlp.2.weight']) * (c['z0'] > 0)
    g['color_predictor.mlp.0.weight'] = dz0.T @ c['x']
    g['color_predictor.mlp.0.bias'] = dz0.sum(0)
    dx = dz0 @ p['color_predictor.mlp.0.weight']
    nf = spec.F * (2 * spec.Lf + 1)
    f = c['f']
    df = dx[:, :spec.F].copy()
    for k in range(spec.Lf):
        s = dt(2.0 ** k)
        gs = dx[:, spec.F * (1 + 2 * k):spec.F * (2 + 2 * k)]
        gc = dx[:, spec.F * (2 + 2 * k):spec.F * (3 + 2 * k)]
        df += s * (gs * np.cos(f * s) - gc * np.sin(f * s))
    del nf
    g['basis_matrix_color.weight'] = df.T @ c['f144']
    return g, df @ p['basis_matrix_color.weight']


def tensorf_forward(tp, spec, rays_o, rays_d, z, *, alpha_vol=None, alpha_bbox=None, distance_scale=25.0,
                    weight_threshold=1e-4, white=False, density='relu', density_offset=-10.0, world_rays=None):
    """LowRankTensor.forward (SimpleTensoRF09.py:701-761), VM (or CP) decomposition.

    tp: dict with 'bbox' (2,3), 'planes_density'/'lines_density'/'planes_color'/'lines_color'
    (lists of (R,H,W) / (R,L,1)), and renderer params.  z (N,S).
    ``world_rays`` = (rays_o, rays_d) in world space switches to NDC mode: rays_o,
    rays_d and z are then the NDC rays and depths that the samples march along
    (SimpleTensoRF09.py:263-277), and compositing takes its deltas from the NDC
    rays and converts depths with the world rays (:779-797).
    Returns the output dict plus a cache for :func:`tensorf_backward`.
    """
    n, s = z.shape
    dt = rays_o.dtype.type
    bbox = tp['bbox']
    pts = rays_o[:, None, :] + rays_d[:, None, :] * z[:, :, None]
    valid = np.all((bbox[0] <= pts) & (pts <= bbox[1]), -1)
    if alpha_vol is not None:
        flat = pts.reshape(-1, 3)
        vidx = np.nonzero(valid.reshape(-1))[0]
        ok = grid_sample_3d_positive(alpha_vol, normalize_points(flat[vidx], alpha_bbox))
        vm = valid.reshape(-1).copy()
        vm[vidx] = ok
        valid = vm.reshape(n, s)
    pn = normalize_points(pts, bbox).reshape(-1, 3)
    vflat = np.nonzero(valid.reshape(-1))[0]
    cp = 'planes_density' not in tp   # CP decomposition: lines only (SimpleTensoRF09.py:964-1123)
    if cp:
        sig_feat = cp_density(tp['lines_density'], pn[vflat])
    else:
        sig_feat = vm_density(tp['planes_density'], tp['lines_density'], pn[vflat])
    if density == 'relu':
        sig_v = relu(sig_feat)
    else:
        xx = sig_feat + dt(density_offset)
        sig_v = np.log1p(np.exp(-np.abs(xx))) + np.maximum(xx, dt(0))
    sigma = np.zeros(n * s, dtype=rays_o.dtype)
    sigma[vflat] = sig_v
    sigma = sigma.reshape(n, s)
    rgb0 = np.zeros((n, s, 3), dtype=rays_o.dtype)
    if world_rays is None:
        out, cc = composite_forward(sigma, rgb0, z, rays_d, distance_scale=distance_scale)
    else:
        out, cc = composite_forward(sigma, rgb0, z, world_rays[1], ndc=True, rays_o=world_rays[0],
                                    rays_d_ndc=rays_d, distance_scale=distance_scale)
    surf = out['weights'] > dt(weight_threshold)
    sflat = np.nonzero(surf.reshape(-1))[0]
    if cp:
        feats = cp_lines(tp['lines_color'], pn[sflat])
        f144 = (feats[0] * feats[1] * feats[2]).T
    else:
        feats = vm_features(tp['planes_color'], tp['lines_color'], pn[sflat])
        f144 = np.concatenate([(pc * lc) for pc, lc in feats], 0).T
    vd = np.repeat(rays_d / np.sqrt(np.sum(rays_d * rays_d, -1, keepdims=True)), s, axis=0)[sflat]
    rgb_s, rc = renderer_forward(tp, spec, f144, vd)
    rgb = np.zeros((n * s, 3), dtype=rays_o.dtype)
    rgb[sflat] = rgb_s
    rgb = rgb.reshape(n, s, 3)
    rgb_map = np.sum(out['weights'][..., None] * rgb, -2)
    if white:
        rgb_map = rgb_map + (dt(1) - out['acc'][:, None])
    out = dict(out)
    out['rgb'] = rgb_map
    out['raw_sigma'] = sigma[..., None]
    out['raw_rgb'] = rgb
    cc['rgb'] = rgb
    cc['white_bkgd'] = white
    cache = dict(cc=cc, pn=pn, vflat=vflat, sflat=sflat, sig_feat=sig_feat, feats=feats, rc=rc,
                 density=density, density_offset=density_offset, n=n, s=s, cp=cp)
    return out, cache


def tensorf_backward(tp, spec, cache, g):
    """Gradients of the VM planes/lines and renderer params for output gradients ``g``."""
    cc = cache['cc']
    dsig, drgb = composite_backward(cc, g)
    n, s = cache['n'], cache['s']
    dt = dsig.dtype.type
    pn, vflat, sflat = cache['pn'], cache['vflat'], cache['sflat']
    grads = {}
    drgb_s = drgb.reshape(-1, 3)[sflat]
    gr, df144 = renderer_backward(tp, spec, cache['rc'], drgb_s)
    grads.update(gr)
    pp = pn[sflat]
    if cache['cp']:
        ls = cache['feats']
        d = df144.T
        for i in range(3):
            v = VECTOR_AXES[i]
            others = ls[(i + 1) % 3] * ls[(i + 2) % 3]
            grads[f'lines_color.{i}'] = grid_sample_2d_backward(tp['lines_color'][i].shape, np.zeros_like(pp[:, v]),
                                                                pp[:, v], d * others, dt)
    off = 0
    for i in range(0 if cache['cp'] else 3):
        m0, m1 = MATRIX_AXES[i]
        v = VECTOR_AXES[i]
        pc, lc = cache['feats'][i]
        r = pc.shape[0]
        d = df144[:, off:off + r].T
        off += r
        grads[f'planes_color.{i}'] = grid_sample_2d_backward(tp['planes_color'][i].shape, pp[:, m0], pp[:, m1], d * lc, dt)
        grads[f'lines_color.{i}'] = grid_sample_2d_backward(tp['lines_color'][i].shape, np.zeros_like(pp[:, v]), pp[:, v], d * pc, dt)
    ds = dsig.reshape(-1)[vflat]
    sf = cache['sig_feat']
    if cache['density'] == 'relu':
        dfeat = ds * (sf > 0)
    else:
        xx = sf + dt(cache['density_offset'])
        dfeat = ds * sigmoid(xx)
    pv = pn[vflat]
    if cache['cp']:
        ls = cp_lines(tp['lines_density'], pv)
        for i in range(3):
            v = VECTOR_AXES[i]
            others = ls[(i + 1) % 3] * ls[(i + 2) % 3]
            grads[f'lines_density.{i}'] = grid_sample_2d_backward(tp['lines_density'][i].shape,
                                                                  np.zeros_like(pv[:, v]), pv[:, v],
                                                                  dfeat[None, :] * others, dt)
        return grads
    feats = vm_features(tp['planes_density'], tp['lines_density'], pv)
    for i in range(3):
        m0, m1 = MATRIX_AXES[i]
        v = VECTOR_AXES[i]
        pc, lc = feats[i]
        grads[f'planes_density.{i}'] = grid_sample_2d_backward(tp['planes_density'][i].shape, pv[:, m0], pv[:, m1], dfeat[None, :] * lc, dt)
        grads[f'lines_density.{i}'] = grid_sample_2d_backward(tp['lines_density'][i].shape, np.zeros_like(pv[:, v]), pv[:, v], dfeat[None, :] * pc, dt)
    return grads


def seeded_vm_model(seed, res, n_density, n_color, features, units, views_pe=2, features_pe=2, scale=0.1):
    """Parameters of a VM model from a numpy PCG64 seed (fixtures regenerate them
    instead of storing them): planes (R, res[m1], res[m0]) and lines (R, res[v], 1)
    ~ N(0, scale^2) as VmDecomposedTensor.create_decomposed_tensor draws them
    (SimpleTensoRF09.py:1154-1165), the basis and renderer layers uniform in
    +-1/sqrt(fan_in) as torch.nn.Linear's default, the last bias zero (:1393)."""
    rng = np.random.default_rng(seed)
    tp = {}
    for kind, comps in (('density', n_density), ('color', n_color)):
        tp[f'planes_{kind}'], tp[f'lines_{kind}'] = [], []
        for i in range(3):
            m0, m1 = MATRIX_AXES[i]
            v = VECTOR_AXES[i]
            tp[f'planes_{kind}'].append(rng.standard_normal((comps[i], res[m1], res[m0]), dtype=np.float32) *
                                        np.float32(scale))
            tp[f'lines_{kind}'].append(rng.standard_normal((comps[i], res[v], 1), dtype=np.float32) * np.float32(scale))
    spec = RendererSpec(features_dim=features, features_pe=features_pe, views_pe=views_pe, units=units)
    shapes = spec.param_shapes(sum(n_color))
    for name, shape in shapes.items():
        # a bias takes the fan-in of its layer's weight
        fan_in = shapes[name.replace('.bias', '.weight')][1]
        b = 1.0 / np.sqrt(fan_in)
        tp[name] = rng.uniform(-b, b, shape).astype(np.float32)
    tp['color_predictor.mlp.4.bias'][:] = 0
    return tp, spec
