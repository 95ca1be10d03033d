"""Numpy restatement of the Simple-NeRF rendering path -- TEST INFRASTRUCTURE ONLY.

Every function follows one reference function (cited file:line, paths relative
to the reference project root).  Forward passes are formula-identical to the
reference; backward passes are derived by hand (the reference relies on torch
autograd) and are checked against the reference's autograd gradients by the
golden fixtures and against central finite differences in float64.

All functions take a ``dtype`` implicitly from their inputs, so the same code
gives the float32 parity oracle and the float64 error oracle.

Where torch's CPU kernels accumulate in double (``cumsum``/``cumprod``:
``at::acc_type<float, false>`` is double), the restatement does the same and
rounds each output once, so the float32 oracle tracks the reference closely.
"""
import numpy as np

# ----------------------------------------------------------------------------
# small helpers
# ----------------------------------------------------------------------------


def torch_linspace(start, end, steps, dtype=np.float32):
    """torch.linspace's CPU formula: the first half counts up from ``start``,
    the second half counts down from ``end`` (symmetric rounding)."""
    out = np.empty(steps, dtype=dtype)
    if steps == 0:
        return out
    if steps == 1:
        out[0] = start
        return out
    dt = np.dtype(dtype).type
    start = dt(start)
    end = dt(end)
    step = dt((end - start) / dt(steps - 1))
    half = steps // 2
    for i in range(steps):
        if i < half:
            out[i] = start + step * dt(i)
        else:
            out[i] = end - step * dt(steps - i - 1)
    return out


def _cumsum(x):
    """torch CPU cumsum: running sum in double, each output rounded once."""
    return np.cumsum(x.astype(np.float64), axis=-1).astype(x.dtype)


def _cumprod(x):
    """torch CPU cumprod: running product in double, each output rounded once."""
    return np.cumprod(x.astype(np.float64), axis=-1).astype(x.dtype)


def relu(x):
    return np.maximum(x, x.dtype.type(0))


def sigmoid(x):
    one = x.dtype.type(1)
    return one / (one + np.exp(-x))


# ----------------------------------------------------------------------------
# rays  (src/utils/CommonUtils04.py)
# ----------------------------------------------------------------------------


def ndc_rays(rays_o, rays_d, h, w, fx, fy, near):
    """CommonUtils04.py:120-138 get_ndc_rays_tr.  ``fx``/``fy`` per ray (N,)."""
    dt = rays_o.dtype.type
    t = -(dt(near) + rays_o[:, 2]) / rays_d[:, 2]
    o = rays_o + t[:, None] * rays_d
    o0 = dt(-1.) / (dt(w) / (dt(2.) * fx)) * o[:, 0] / o[:, 2]
    o1 = dt(-1.) / (dt(h) / (dt(2.) * fy)) * o[:, 1] / o[:, 2]
    o2 = dt(1.) + dt(2.) * dt(near) / o[:, 2]
    d0 = dt(-1.) / (dt(w) / (dt(2.) * fx)) * (rays_d[:, 0] / rays_d[:, 2] - o[:, 0] / o[:, 2])
    d1 = dt(-1.) / (dt(h) / (dt(2.) * fy)) * (rays_d[:, 1] / rays_d[:, 2] - o[:, 1] / o[:, 2])
    d2 = dt(-2.) * dt(near) / o[:, 2]
    return np.stack([o0, o1, o2], -1), np.stack([d0, d1, d2], -1)


def view_dirs(rays_d):
    """CommonUtils04.py:147-149 get_view_dirs_tr."""
    return rays_d / np.sqrt(np.sum(rays_d * rays_d, -1, keepdims=True))


def rays_from_pixels(pixel_id, intrinsics, extrinsics, half_pixel=False):
    """CommonUtils04.py:73-95 get_rays_tr (non-synthetic branch).

    pixel_id (N,3) int (image, x, y); intrinsics (N,3,3); extrinsics (N,4,4) c2w.
    """
    dt = intrinsics.dtype
    x = pixel_id[:, 1].astype(dt)
    y = pixel_id[:, 2].astype(dt)
    if half_pixel:
        x = x + dt.type(0.5)
        y = y + dt.type(0.5)
    pts = np.stack([x, y, np.ones_like(x)], 1)
    kinv = np.linalg.inv(intrinsics.astype(np.float64)).astype(dt)
    dirs = np.einsum('nij,nj->ni', kinv, pts)
    dirs[:, 1:] *= -1
    rays_d = np.sum(dirs[:, None, :] * extrinsics[:, :3, :3], -1)
    rays_o = extrinsics[:, :3, 3].copy()
    return rays_o, rays_d


# ----------------------------------------------------------------------------
# sampling  (src/models/SimpleNeRF17.py)
# ----------------------------------------------------------------------------


def stratified_z(near, far, n_rays, n_samples, u=None, lindisp=False, dtype=np.float32):
    """SimpleNeRF17.py:330-358 get_z_vals_coarse.  ``u`` (N,S) uniforms, None = no jitter."""
    dt = np.dtype(dtype).type
    t = torch_linspace(0., 1., n_samples, dtype)
    if not lindisp:
        z = dt(near) * (dt(1.) - t) + dt(far) * t
    else:
        z = dt(1.) / (dt(1.) / dt(near) * (dt(1.) - t) + dt(1.) / dt(far) * t)
    z = np.broadcast_to(z, (n_rays, n_samples)).copy()
    if u is not None:
        mids = dt(.5) * (z[:, 1:] + z[:, :-1])
        upper = np.concatenate([mids, z[:, -1:]], -1)
        lower = np.concatenate([z[:, :1], mids], -1)
        z = lower + (upper - lower) * u.astype(dtype)
    return z


def searchsorted_right(cdf, u):
    """torch.searchsorted(cdf, u, right=True) on sorted rows: count of cdf <= u."""
    return np.sum(cdf[:, None, :] <= u[:, :, None], axis=-1)


def sample_pdf(bins, weights, n_samples, u=None):
    """SimpleNeRF17.py:384-417 sample_pdf (identical copy SimpleTensoRF09.py:427-460).

    bins (N,B), weights (N,B-1), u (N,n) uniforms or None for the deterministic
    linspace(0,1,n) used when perturbation is off.
    """
    dtype = weights.dtype
    dt = dtype.type
    w = weights + dt(1e-5)
    pdf = w / np.sum(w, -1, keepdims=True)
    cdf = _cumsum(pdf)
    cdf = np.concatenate([np.zeros_like(cdf[:, :1]), cdf], -1)
    n = cdf.shape[0]
    if u is None:
        u = np.broadcast_to(torch_linspace(0., 1., n_samples, dtype), (n, n_samples))
    u = np.ascontiguousarray(u, dtype=dtype)
    inds = searchsorted_right(cdf, u)
    below = np.maximum(0, inds - 1)
    above = np.minimum(cdf.shape[-1] - 1, inds)
    rows = np.arange(n)[:, None]
    cdf0, cdf1 = cdf[rows, below], cdf[rows, above]
    bins0, bins1 = bins[rows, below], bins[rows, above]
    denom = cdf1 - cdf0
    denom = np.where(denom < dt(1e-5), dt(1.), denom)
    t = (u - cdf0) / denom
    return bins0 + t * (bins1 - bins0)


def fine_z(z_coarse, weights_coarse, n_fine, u=None):
    """SimpleNeRF17.py:360-371 get_z_vals_fine: pdf samples merged and sorted with z_coarse."""
    mids = z_coarse.dtype.type(.5) * (z_coarse[:, 1:] + z_coarse[:, :-1])
    samples = sample_pdf(mids, weights_coarse[:, 1:-1], n_fine, u)
    return np.sort(np.concatenate([z_coarse, samples], -1), -1, kind='stable')


# ----------------------------------------------------------------------------
# positional encoding + MLP  (src/models/SimpleNeRF17.py:581-785)
# ----------------------------------------------------------------------------


def positional_encoding(x, degree):
    """SimpleNeRF17.py:581-613 + 669-682: [x, sin(2^0 x), cos(2^0 x), ..., sin(2^{L-1} x), cos(2^{L-1} x)]."""
    dt = x.dtype.type
    parts = [x]
    for k in range(degree):
        xf = x * dt(2.0 ** k)
        parts.append(np.sin(xf))
        parts.append(np.cos(xf))
    return np.concatenate(parts, -1)


def positional_encoding_backward(x, degree, grad):
    """d/dx of positional_encoding (only needed by tests of the encoder alone)."""
    dt = x.dtype.type
    d = x.shape[-1]
    gx = grad[..., :d].copy()
    for k in range(degree):
        f = dt(2.0 ** k)
        xf = x * f
        gs = grad[..., d * (1 + 2 * k):d * (2 + 2 * k)]
        gc = grad[..., d * (2 + 2 * k):d * (3 + 2 * k)]
        gx += f * (gs * np.cos(xf) - gc * np.sin(xf))
    return gx


class MlpSpec:
    """Architecture of one reference ``MLP`` (SimpleNeRF17.py:616-667)."""

    def __init__(self, points_net_depth=8, points_net_width=256, views_net_depth=1, views_net_width=128,
                 points_pe_degree=10, views_pe_degree=4, use_view_dirs=True, view_dependent_rgb=True,
                 points_sigma_pe_degree=None):
        self.Dp, self.Wp, self.Dv, self.Wv = points_net_depth, points_net_width, views_net_depth, views_net_width
        self.Lp, self.Lv = points_pe_degree, views_pe_degree
        self.use_view_dirs = use_view_dirs
        self.view_dep_rgb = view_dependent_rgb
        self.Lps = points_sigma_pe_degree
        self.pts_pe_dim = 3 * (2 * self.Lp + 1)
        self.pts_input_dim = self.pts_pe_dim if self.Lps is None else 3 * (2 * self.Lps + 1)
        self.views_input_dim = 3 * (2 * self.Lv + 1) if use_view_dirs else 0
        if self.Lps is not None:
            self.views_input_dim += self.pts_pe_dim - self.pts_input_dim
        self.skips = [4]
        self.view_dep_outputs = self.view_dep_rgb

    @classmethod
    def from_config(cls, c):
        return cls(c['points_net_depth'], c['points_net_width'], c['views_net_depth'], c['views_net_width'],
                   c['points_positional_encoding_degree'], c.get('views_positional_encoding_degree', 0),
                   c['use_view_dirs'], c['view_dependent_rgb'], c.get('points_sigma_positional_encoding_degree'))

    def param_shapes(self):
        """Parameter names and shapes exactly as the reference's state_dict keys."""
        s = {}
        s['pts_linears.0.weight'] = (self.Wp, self.pts_input_dim)
        s['pts_linears.0.bias'] = (self.Wp,)
        for j in range(1, self.Dp):
            k_in = self.Wp + self.pts_input_dim if (j - 1) in self.skips else self.Wp
            s[f'pts_linears.{j}.weight'] = (self.Wp, k_in)
            s[f'pts_linears.{j}.bias'] = (self.Wp,)
        if self.view_dep_outputs:
            s['views_linears.0.weight'] = (self.Wv, self.views_input_dim + self.Wp)
            s['views_linears.0.bias'] = (self.Wv,)
            for j in range(1, self.Dv):
                s[f'views_linears.{j}.weight'] = (self.Wv, self.Wv)
                s[f'views_linears.{j}.bias'] = (self.Wv,)
        s['pts_output_linear.weight'] = (1 if self.view_dep_rgb else 4, self.Wp)
        s['pts_output_linear.bias'] = (1 if self.view_dep_rgb else 4,)
        if self.view_dep_outputs:
            s['feature_linear.weight'] = (self.Wp, self.Wp)
            s['feature_linear.bias'] = (self.Wp,)
            s['views_output_linear.weight'] = (3, self.Wv)
            s['views_output_linear.bias'] = (3,)
        return s

    def macs_per_sample(self):
        return sum(int(np.prod(v)) for k, v in self.param_shapes().items() if k.endswith('weight'))


def xavier_params(spec, seed, dtype=np.float32):
    """Xavier-uniform weights, zero biases, from a numpy PCG64 stream (bit-stable across machines)."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, shape in spec.param_shapes().items():
        if name.endswith('weight'):
            fan_out, fan_in = shape
            bound = np.sqrt(6.0 / (fan_in + fan_out))
            p[name] = rng.uniform(-bound, bound, size=shape).astype(dtype)
        else:
            p[name] = np.zeros(shape, dtype=dtype)
    return p


def mlp_forward(p, spec, pts, vdirs=None, sigma_noise=None):
    """SimpleNeRF17.py:696-785 MLP.forward.  pts (M,3); vdirs (M,3) per sample.

    Returns sigma (M,1), rgb (M,3) and a cache for :func:`mlp_backward`.
    ``sigma_noise`` (M,1) is the already-scaled ``raw_noise_std * randn`` term (:739-741).
    """
    c = {'pts': pts}
    enc = positional_encoding(pts, spec.Lp)
    inp = enc[:, :spec.pts_input_dim]
    h = inp
    ins, zs = [], []
    for i in range(spec.Dp):
        W, b = p[f'pts_linears.{i}.weight'], p[f'pts_linears.{i}.bias']
        ins.append(h)
        z = h @ W.T + b
        zs.append(z)
        h = relu(z)
        if i in spec.skips:
            h = np.concatenate([inp, h], -1)
    c['trunk_in'], c['trunk_z'], c['h'] = ins, zs, h
    out = h @ p['pts_output_linear.weight'].T + p['pts_output_linear.bias']
    sraw = out[:, 0:1]
    if sigma_noise is not None:
        sraw = sraw + sigma_noise
    c['sigma_raw'] = sraw
    sigma = relu(sraw)
    if not spec.view_dep_rgb:
        rgb = sigmoid(out[:, 1:4])
        c['rgb'] = rgb
        return sigma, rgb, c
    feat = h @ p['feature_linear.weight'].T + p['feature_linear.bias']
    feat = np.concatenate([feat, enc[:, spec.pts_input_dim:]], -1)
    ev = positional_encoding(vdirs, spec.Lv)
    hv = np.concatenate([feat, ev], -1)
    vins, vzs = [], []
    for j in range(spec.Dv):
        W, b = p[f'views_linears.{j}.weight'], p[f'views_linears.{j}.bias']
        vins.append(hv)
        z = hv @ W.T + b
        vzs.append(z)
        hv = relu(z)
    c['views_in'], c['views_z'], c['hv'] = vins, vzs, hv
    vo = hv @ p['views_output_linear.weight'].T + p['views_output_linear.bias']
    rgb = sigmoid(vo[:, 0:3])
    c['rgb'] = rgb
    return sigma, rgb, c


def mlp_backward(p, spec, c, dsigma, drgb):
    """Hand-derived adjoint of :func:`mlp_forward` w.r.t. every parameter."""
    g = {}
    dt = dsigma.dtype.type
    rgb = c['rgb']
    drgb_pre = drgb * rgb * (dt(1) - rgb)
    dsig_pre = dsigma * (c['sigma_raw'] > 0)
    h = c['h']
    if not spec.view_dep_rgb:
        dout = np.concatenate([dsig_pre, drgb_pre], -1)
        g['pts_output_linear.weight'] = dout.T @ h
        g['pts_output_linear.bias'] = dout.sum(0)
        dh = dout @ p['pts_output_linear.weight']
    else:
        dvo = drgb_pre
        g['views_output_linear.weight'] = dvo.T @ c['hv']
        g['views_output_linear.bias'] = dvo.sum(0)
        dhv = dvo @ p['views_output_linear.weight']
        for j in reversed(range(spec.Dv)):
            dz = dhv * (c['views_z'][j] > 0)
            g[f'views_linears.{j}.weight'] = dz.T @ c['views_in'][j]
            g[f'views_linears.{j}.bias'] = dz.sum(0)
            dhv = dz @ p[f'views_linears.{j}.weight']
        dfeat = dhv[:, :spec.Wp]
        g['feature_linear.weight'] = dfeat.T @ h
        g['feature_linear.bias'] = dfeat.sum(0)
        dh = dfeat @ p['feature_linear.weight']
        g['pts_output_linear.weight'] = dsig_pre.T @ h
        g['pts_output_linear.bias'] = dsig_pre.sum(0)
        dh = dh + dsig_pre @ p['pts_output_linear.weight']
    for i in reversed(range(spec.Dp)):
        if i in spec.skips:
            dh = dh[:, spec.pts_input_dim:]
        dz = dh * (c['trunk_z'][i] > 0)
        g[f'pts_linears.{i}.weight'] = dz.T @ c['trunk_in'][i]
        g[f'pts_linears.{i}.bias'] = dz.sum(0)
        dh = dz @ p[f'pts_linears.{i}.weight']
    return g


# ----------------------------------------------------------------------------
# compositing  (SimpleNeRF17.py:486-558, SimpleTensoRF09.py:767-819)
# ----------------------------------------------------------------------------


def depth_from_ndc(z_ndc, rays_o, rays_d):
    """SimpleNeRF17.py:541-558 convert_depth_from_ndc (near hard-coded to 1)."""
    dt = z_ndc.dtype.type
    oz = rays_o[:, 2:3]
    dz = rays_d[:, 2:3]
    tn = -(dt(1) + oz) / dz
    const = np.where(z_ndc == dt(1.), dt(1e-3), dt(0.))
    return (oz + tn * dz) / dz * (dt(1) / (dt(1) - z_ndc + const) - dt(1)) + tn


def composite_forward(sigma, rgb, z, rays_d, *, ndc=False, rays_o=None, rays_d_ndc=None,
                      white_bkgd=False, distance_scale=None):
    """SimpleNeRF17.py:486-539 volume_rendering (distance_scale: SimpleTensoRF09.py:787).

    sigma (N,S), rgb (N,S,3), z (N,S) -- the NDC z when ``ndc``.
    Returns the reference's output dict and a cache for :func:`composite_backward`.
    """
    dt = sigma.dtype.type
    inf_depth = dt(1.) if ndc else dt(1e10)
    z1 = np.concatenate([z, np.full_like(z[:, :1], inf_depth)], -1)
    dists = z1[:, 1:] - z1[:, :-1]
    dvec = rays_d_ndc if ndc else rays_d
    dnorm = np.sqrt(np.sum(dvec * dvec, -1))
    delta = dists * dnorm[:, None]
    x = -sigma * delta
    if distance_scale is not None:
        x = x * dt(distance_scale)
    ex = np.exp(x)
    alpha = dt(1.) - ex
    p = dt(1.) - alpha + dt(1e-10)
    vis = _cumprod(np.concatenate([np.ones_like(p[:, :1]), p], -1))[:, :-1]
    w = alpha * vis
    out = {}
    rgb_map = np.sum(w[..., None] * rgb, -2)
    acc = np.sum(w, -1)
    eps = dt(1e-6)
    if not ndc:
        zm = z
    else:
        dndc = np.sum(w * z, -1) / (acc + eps)
        out['depth_ndc'] = dndc
        out['depth_var_ndc'] = np.sum(w * np.square(z - dndc[:, None]), -1)
        zm = depth_from_ndc(z, rays_o, rays_d)
    depth = np.sum(w * zm, -1) / (acc + eps)
    out['depth_var'] = np.sum(w * np.square(zm - depth[:, None]), -1)
    out['depth'] = depth
    if white_bkgd:
        rgb_map = rgb_map + (dt(1.) - acc[:, None])
    out.update({'rgb': rgb_map, 'acc': acc, 'alpha': alpha, 'visibility': vis, 'weights': w})
    cache = dict(sigma=sigma, rgb=rgb, z=z, zm=zm, delta=delta, ex=ex, alpha=alpha, p=p, vis=vis, w=w,
                 acc=acc, ndc=ndc, white_bkgd=white_bkgd, ds=distance_scale, out=out)
    return out, cache


def composite_backward(cache, g):
    """Adjoint of :func:`composite_forward`.

    ``g`` maps output names (rgb, acc, depth, depth_var, depth_ndc, depth_var_ndc,
    weights) to upstream gradients; missing entries are zero.  Returns
    (dsigma (N,S), drgb (N,S,3)).  The transmittance adjoint is a reverse linear
    recurrence R_i = G_{i+1} a_{i+1} + p_{i+1} R_{i+1} (no division by p).
    """
    w, acc, rgb = cache['w'], cache['acc'], cache['rgb']
    dt = w.dtype.type
    n, s = w.shape
    eps = dt(1e-6)
    out = cache['out']
    zero_n = np.zeros(n, dtype=w.dtype)
    g_rgb = g.get('rgb', np.zeros((n, 3), dtype=w.dtype))
    g_acc = g.get('acc', zero_n).copy()
    if cache['white_bkgd']:
        g_acc = g_acc - np.sum(g_rgb, -1)
    G = np.sum(rgb * g_rgb[:, None, :], -1) + g_acc[:, None]
    if 'weights' in g:
        G = G + g['weights']

    def depth_terms(zz, dep, gd, gv):
        r = zz - dep[:, None]
        b = np.sum(w * r, -1)
        return gd[:, None] * r / (acc + eps)[:, None] + gv[:, None] * (r * r - dt(2) * b[:, None] * r / (acc + eps)[:, None])

    G = G + depth_terms(cache['zm'], out['depth'], g.get('depth', zero_n), g.get('depth_var', zero_n))
    if cache['ndc']:
        G = G + depth_terms(cache['z'], out['depth_ndc'], g.get('depth_ndc', zero_n), g.get('depth_var_ndc', zero_n))
    alpha, p, vis = cache['alpha'], cache['p'], cache['vis']
    R = np.zeros_like(w)
    for i in range(s - 2, -1, -1):
        R[:, i] = G[:, i + 1] * alpha[:, i + 1] + p[:, i + 1] * R[:, i + 1]
    dalpha = G * vis - vis * R
    dx = -dalpha * cache['ex']
    if cache['ds'] is not None:
        dx = dx * dt(cache['ds'])
    dsigma = -dx * cache['delta']
    drgb = w[..., None] * g_rgb[:, None, :]
    return dsigma, drgb


# ----------------------------------------------------------------------------
# whole-path drivers (the 1024-ray render, the 4096-ray train step)
# ----------------------------------------------------------------------------


def render_rays(params_c, params_f, spec_c, spec_f, rays_o, rays_d, near, far, n_coarse, n_fine,
                u_coarse=None, u_fine=None, white_bkgd=False, ndc=None, aug=None, z_fine=None, pts_fp32=False):
    """SimpleNeRF17.py:159-328 render_rays for synthetic rays (ray generation patched out).

    ``ndc`` = dict(h, w, fx, fy, near) switches to NDC rays (the main + augmented pair).  ``aug`` =
    list of (name, params, spec) augmented coarse nets run on the coarse samples
    (:244-261) and, when they also carry fine params, on the fine samples (:296-313).
    ``z_fine`` (N, Sc+Sf) replaces the inverse-CDF depths (tests use it to check
    the fine pass on exactly the depths another implementation sampled).
    ``pts_fp32`` forms the sample positions in float32 (product, then sum, as the
    reference's two torch ops do at :213-215) before the network sees them, so a
    float64 evaluation shares the float32 input quantisation of any float32
    implementation: PE scales that rounding by up to 2^9.
    Returns (outputs dict keyed like the reference, caches for backward).
    """
    ret, caches = {}, {}
    n = rays_o.shape[0]
    if ndc is not None:
        o_ndc, d_ndc = ndc_rays(rays_o, rays_d, ndc['h'], ndc['w'], ndc['fx'], ndc['fy'], ndc['near'])
        po, pd = o_ndc, d_ndc
    else:
        o_ndc = d_ndc = None
        po, pd = rays_o, rays_d
    vd = view_dirs(rays_d)
    zc = stratified_z(near, far, n, n_coarse, u_coarse, dtype=rays_o.dtype)

    def run(params, spec, z, tag):
        s = z.shape[1]
        if pts_fp32:
            f = np.float32
            pts = (po.astype(f)[:, None, :] + pd.astype(f)[:, None, :] * z.astype(f)[:, :, None])
            pts = pts.reshape(-1, 3).astype(z.dtype)
        else:
            pts = (po[:, None, :] + pd[:, None, :] * z[:, :, None]).reshape(-1, 3)
        vds = np.repeat(vd, s, axis=0) if spec.use_view_dirs else None
        sigma, rgb, mc = mlp_forward(params, spec, pts, vds)
        sigma = sigma.reshape(n, s)
        rgb = rgb.reshape(n, s, 3)
        out, cc = composite_forward(sigma, rgb, z, rays_d, ndc=ndc is not None, rays_o=rays_o,
                                    rays_d_ndc=d_ndc, white_bkgd=white_bkgd)
        caches[tag] = (mc, cc)
        return out, sigma, rgb

    out_c, sc, rc = run(params_c, spec_c, zc, 'coarse')
    ret['z_vals_coarse'] = zc
    for k, v in out_c.items():
        ret[f'{k}_coarse'] = v
    ret['raw_sigma_coarse'], ret['raw_rgb_coarse'] = sc[..., None], rc
    for name, prm, spc in (aug or []):
        o, _, _ = run(prm['coarse'], spc, zc, f'{name}_coarse')
        for k, v in o.items():
            ret[f'{name}_{k}_coarse'] = v
    if params_f is not None:
        zf = fine_z(zc, out_c['weights'], n_fine, u_fine) if z_fine is None else z_fine.astype(zc.dtype)
        out_f, sf, rf = run(params_f, spec_f, zf, 'fine')
        ret['z_vals_fine'] = zf
        for k, v in out_f.items():
            ret[f'{k}_fine'] = v
        ret['raw_sigma_fine'], ret['raw_rgb_fine'] = sf[..., None], rf
        for name, prm, spc in (aug or []):
            if prm.get('fine') is not None:
                o, _, _ = run(prm['fine'], spc, zf, f'{name}_fine')
                for k, v in o.items():
                    ret[f'{name}_{k}_fine'] = v
    return ret, caches


def train_loss(ret, target_rgb, target_depth, depth_mask, depth_weight=0.1, nets=('coarse', 'fine')):
    """Training loss of the 4096-ray training step: per net, MSE(rgb, target) (MSE14.py:81-94
    form: mean over channels then rays) + depth_weight * mean |depth - target| over
    the depth-supervised rays.  Returns (loss, {output_key: grad})."""
    dt = target_rgb.dtype.type
    loss = 0.0
    grads = {}
    n = target_rgb.shape[0]
    nd = int(depth_mask.sum())
    for tag in nets:
        err = ret[f'rgb_{tag}'] - target_rgb
        loss += float(np.mean(np.mean(err * err, 1)))
        grads[f'rgb_{tag}'] = (dt(2.0) / dt(3 * n)) * err
        de = ret[f'depth_{tag}'] - target_depth
        loss += depth_weight * float(np.sum(np.abs(de) * depth_mask) / max(nd, 1))
        grads[f'depth_{tag}'] = (dt(depth_weight) / dt(max(nd, 1))) * np.sign(de) * depth_mask
    return loss, grads


def backward_render(params, specs, caches, grads, n_rays):
    """Parameter gradients of a loss whose output-gradients are ``grads`` (keys like
    ``rgb_coarse``/``depth_fine``), through composite and MLP adjoints.  No gradient
    flows through the sampling (SimpleNeRF17.py:368 detaches the fine z)."""
    out = {}
    for tag, (mc, cc) in caches.items():
        g = {}
        for k in ('rgb', 'acc', 'depth', 'depth_var', 'depth_ndc', 'depth_var_ndc', 'weights'):
            if f'{k}_{tag}' in grads:
                g[k] = grads[f'{k}_{tag}']
        if not g:
            continue
        dsig, drgb = composite_backward(cc, g)
        out[tag] = mlp_backward(params[tag], specs[tag], mc, dsig.reshape(-1, 1), drgb.reshape(-1, 3))
    return out
