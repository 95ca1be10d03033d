"""Central finite differences in float64 of the training-step loss -- TEST
INFRASTRUCTURE ONLY.

The reference differentiates with torch autograd (Trainer10.py:103
``TotalLoss.backward()``); the sample depths carry no gradient (the fine depths
are detached, SimpleNeRF17.py:368).  These helpers evaluate one net's share of
the training loss at FIXED sample depths, so a central difference along a
parameter direction v,

    (L(p + eps v) - L(p - eps v)) / (2 eps),

is the directional derivative that the hand-written backward (oracle or GPU)
must reproduce as <grad, v>.  Every evaluation is float64 numpy.
"""
import numpy as np

from . import nerf as on


def level_loss(params, spec, rays_o, rays_d, z, target_rgb, target_depth, depth_mask, *, white_bkgd=True,
               depth_weight=0.1):
    """One net's share of the training step's loss at fixed depths ``z`` (N, S):
    MSE(rgb, target) (MSE14.py:81-94) + depth_weight * mean L1 depth on the
    depth-supervised rays, rendered as SimpleNeRF17.py:486-539 does.

    The sample positions are formed in float32 (product, then sum, as the
    reference's torch ops at SimpleNeRF17.py:213-215 and the GPU kernels do) and
    then widened, so the float64 evaluation shares their input quantisation."""
    n, s = z.shape
    f = np.float32
    pts = (rays_o.astype(f)[:, None, :] + rays_d.astype(f)[:, None, :] * z.astype(f)[:, :, None])
    pts = pts.reshape(-1, 3).astype(np.float64)
    vd = np.repeat(on.view_dirs(rays_d.astype(np.float64)), s, axis=0) if spec.use_view_dirs else None
    sigma, rgb, _ = on.mlp_forward(params, spec, pts, vd)
    out, _ = on.composite_forward(sigma.reshape(n, s), rgb.reshape(n, s, 3), z.astype(np.float64),
                                  rays_d.astype(np.float64), white_bkgd=white_bkgd)
    loss, _ = on.train_loss({'rgb_x': out['rgb'], 'depth_x': out['depth']}, target_rgb.astype(np.float64),
                            target_depth.astype(np.float64), depth_mask.astype(np.float64), depth_weight,
                            nets=('x',))
    return loss


def directional_derivative(loss_fn, params, direction, eps):
    """Central difference of ``loss_fn(params)`` along ``direction`` (a dict with
    a subset of ``params``' keys); ``params`` is left unchanged."""
    plus = dict(params)
    minus = dict(params)
    for k, v in direction.items():
        plus[k] = params[k] + eps * v
        minus[k] = params[k] - eps * v
    return (loss_fn(plus) - loss_fn(minus)) / (2.0 * eps)


def dot(grads, direction):
    """<grads, direction> over the keys of ``direction``, in float64."""
    return float(sum(np.sum(np.asarray(grads[k], np.float64) * v) for k, v in direction.items()))


def unit_directions(ref_grads, keys, rng):
    """Test directions for one net: the whole reference gradient, each named
    tensor's own gradient, and one random Gaussian direction over every tensor --
    each scaled to unit L2 norm."""
    out = []

    def unit(d):
        nrm = np.sqrt(sum(float(np.sum(v * v)) for v in d.values()))
        return {k: v / nrm for k, v in d.items()}

    out.append(('whole gradient', unit({k: np.asarray(v, np.float64) for k, v in ref_grads.items()})))
    for k in keys:
        out.append((k, unit({k: np.asarray(ref_grads[k], np.float64)})))
    out.append(('random', unit({k: rng.standard_normal(np.shape(v)) for k, v in ref_grads.items()})))
    return out
