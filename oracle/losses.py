"""CPU restatement (numpy) of the reference's per-ray training losses whose
gradients feed the compositing adjoint.  Test infrastructure only: the product
path never imports this module.

Each function returns (loss, gradients) for the loss as the reference computes
it on one batch, the gradients being those autograd would give.
"""
import numpy as np

from .nerf import torch_linspace


def depth_mse(pred, target, mask=None, mean_over_mask=False, target_grad=False):
    """Squared depth error of three reference losses:

    * AugmentationsDepthLoss11.compute_depth_mse
      (src/loss_functions/AugmentationsDepthLoss11.py:208-226): entries outside the
      mask set to 0 in both tensors, then the mean over all rays; the target is
      detached by the caller (:187-188).
    * SparseDepthMSE14.compute_depth_loss (src/loss_functions/SparseDepthMSE14.py:84-97):
      pred[mask] - true[mask], mean over the masked rays (``mean_over_mask``).
    * CoarseFineConsistencyLoss33.compute_loss
      (src/loss_functions/CoarseFineConsistencyLoss33.py:35-44): mean over all
      rays of (coarse - fine)^2 with gradients into both (``target_grad``).

    Returns (loss, d loss / d pred, d loss / d target or None).
    """
    pred = np.asarray(pred)
    dt = pred.dtype.type
    m = np.ones(pred.shape, bool) if mask is None else np.asarray(mask, bool)
    e = np.where(m, pred - target, dt(0))
    n = int(m.sum()) if mean_over_mask else pred.shape[0]
    if n == 0:
        return 0.0, np.zeros_like(pred), (np.zeros_like(pred) if target_grad else None)
    loss = float(np.sum(e * e) / n)
    g = (dt(2) / dt(n)) * e
    return loss, g, (-g if target_grad else None)


def bin_sizes(n_samples, num_bins):
    """MassConcentrationLoss06.compute_entropy_loss bin layout (:69-72): S // B samples
    per bin, one more in the bins torch.linspace(0, B-1, S % B).long() selects."""
    per, rem = n_samples // num_bins, n_samples % num_bins
    bigger = set(int(v) for v in torch_linspace(0.0, float(num_bins - 1), rem)) if rem else set()
    return [per + 1 if b in bigger else per for b in range(num_bins)]


def mass_concentration(weights, num_bins, mask=None):
    """MassConcentrationLoss06.compute_entropy_loss
    (src/loss_functions/MassConcentrationLoss06.py:63-83): per ray, sums of the
    weights over contiguous bins, entr(b + 1e-3) = -(b + 1e-3) ln(b + 1e-3) summed
    over bins, mean over the masked rays.  Returns (loss, d loss / d weights)."""
    w = np.asarray(weights)
    dt = w.dtype.type
    n, s = w.shape
    m = np.ones(n, bool) if mask is None else np.asarray(mask, bool)
    sizes = bin_sizes(s, num_bins)
    edges = np.concatenate([[0], np.cumsum(sizes)])
    b = np.stack([w[:, edges[i]:edges[i + 1]].sum(1) for i in range(num_bins)], 1) + dt(1e-3)
    per_ray = -np.sum(b * np.log(b), 1)
    cnt = int(m.sum())
    if cnt == 0:
        return 0.0, np.zeros_like(w)
    loss = float(per_ray[m].sum() / cnt)
    gb = -(np.log(b) + dt(1)) / dt(cnt)
    g = np.zeros_like(w)
    for i in range(num_bins):
        g[:, edges[i]:edges[i + 1]] = gb[:, i:i + 1]
    g[~m] = 0
    return loss, g


def closest_views(poses, image_ids):
    """AugmentationsDepthLoss11.py:134-138: the view whose camera origin is nearest
    to the ray's own camera (second smallest distance, the smallest being the view
    itself).  Ties (two identical origins) are implementation-defined in the
    reference (torch.kthvalue); here the lowest other index wins."""
    o = poses[:, :3, 3].astype(np.float32)
    d = np.sqrt(np.sum(np.square(o[image_ids][:, None, :] - o[None]), -1))
    d[np.arange(len(image_ids)), image_ids] = np.inf
    return np.argmin(d, 1)


def reproject(points, poses_b, k0):
    """CommonUtils04.reproject (src/utils/CommonUtils04.py:227-253): pixel coordinates of
    world points in views poses_b (per point) with the first view's intrinsics k0."""
    f = np.float32
    perm = np.diag(np.array([1, -1, -1], f))
    rt = np.transpose(poses_b[:, :3, :3].astype(f), (0, 2, 1))
    m = (k0.astype(f) @ perm)[None] @ rt
    v = (points.astype(f) - poses_b[:, :3, 3].astype(f))[..., None]
    p = (m @ v)[..., 0]
    return p[:, :2] / p[:, 2:], p


def patch(images, img, y, x, hpy, hpx):
    """(ny, nx, C) patch centred at (y, x) of images[img], zero outside the image
    (the reference pads the end of both axes and lets negative indices wrap onto
    that padding, :158-164)."""
    v, h, w, c = images.shape
    out = np.zeros((2 * hpy + 1, 2 * hpx + 1, c), images.dtype)
    for i, dy in enumerate(range(-hpy, hpy + 1)):
        for j, dx in enumerate(range(-hpx, hpx + 1)):
            yy, xx = y + dy, x + dx
            if 0 <= yy < h and 0 <= xx < w:
                out[i, j] = images[img, yy, xx]
    return out


def reprojection_masks(depth1, depth2, rays_o, rays_d, pixel_ids, poses, k0, images, patch_size=(5, 5),
                       rmse_threshold=0.1, both_invalid_rule=True):
    """AugmentationsDepthLoss11.compute_loss_nerf (src/loss_functions/AugmentationsDepthLoss11.py:105-190)
    on rays that are all NeRF rays: returns (mask1, mask2, pos1, pos2), mask1 where
    depth1 reprojects to the more consistent patch in the nearest other view (so
    depth2 is pulled towards depth1 there) and mask2 the reverse; pos* the
    unrounded reprojected pixel positions (for boundary checks).
    both_invalid_rule=False gives CoarseFineConsistencyLoss34.compute_loss_nerf
    (src/loss_functions/CoarseFineConsistencyLoss34.py:89-168, depth1 coarse,
    depth2 fine), which lacks the rule for rays whose reprojections both leave
    the image (AugmentationsDepthLoss11.py:176-181)."""
    f = np.float32
    v, h, w, _ = images.shape
    hpx, hpy = patch_size[0] // 2, patch_size[1] // 2
    img = pixel_ids[:, 0].astype(np.int64)
    xa, ya = pixel_ids[:, 1].astype(np.int64), pixel_ids[:, 2].astype(np.int64)
    jb = closest_views(poses, img)
    pb = poses[jb]
    p1 = rays_o.astype(f) + rays_d.astype(f) * depth1.astype(f)[:, None]
    p2 = rays_o.astype(f) + rays_d.astype(f) * depth2.astype(f)[:, None]
    pos1, _ = reproject(p1, pb, k0)
    pos2, _ = reproject(p2, pb, k0)
    q1, q2 = np.round(pos1).astype(np.int64), np.round(pos2).astype(np.int64)

    def valid(x, y):
        return (x >= hpx) & (x < w - hpx) & (y >= hpy) & (y < h - hpy)

    va, v1, v2 = valid(xa, ya), valid(q1[:, 0], q1[:, 1]), valid(q2[:, 0], q2[:, 1])
    n = len(img)
    rm1, rm2 = np.zeros(n, f), np.zeros(n, f)
    for r in range(n):
        pa = patch(images, img[r], ya[r], xa[r], hpy, hpx)
        b1 = patch(images, jb[r], int(np.clip(q1[r, 1], 0, h - 1)), int(np.clip(q1[r, 0], 0, w - 1)), hpy, hpx)
        b2 = patch(images, jb[r], int(np.clip(q2[r, 1], 0, h - 1)), int(np.clip(q2[r, 0], 0, w - 1)), hpy, hpx)
        rm1[r] = np.sqrt(np.mean(np.square(pa - b1)))
        rm2[r] = np.sqrt(np.mean(np.square(pa - b2)))
    m1 = ((rm1 < rm2) | ~v2) & (rm1 < rmse_threshold) & v1 & va
    m2 = ((rm2 < rm1) | ~v1) & (rm2 < rmse_threshold) & v2 & va
    if both_invalid_rule:
        both_invalid = ~(v1 | v2)
        m1 |= both_invalid & (depth1 > depth2)
        m2 |= both_invalid & (depth2 > depth1)
    return m1, m2, pos1, pos2


def reprojection_depth_loss(depth1, depth2, mask1, mask2):
    """The loss AugmentationsDepthLoss11.compute_loss_nerf forms from the masks
    (:186-190): compute_depth_mse(depth1, depth2.detach(), mask2) zeroes, in place,
    depth1 and -- through the detached view, which shares its storage -- depth2
    outside mask2; the second term compute_depth_mse(depth2, depth1.detach(), mask1)
    then only sees mask1 & mask2 rays, which the mask rules make disjoint.  So the
    loss is mean_n mask2 (depth1 - depth2)^2 with a gradient into depth1 only.
    Returns (loss, d/d depth1, d/d depth2)."""
    l1, g1, _ = depth_mse(depth1, depth2, mask2)
    both = np.asarray(mask1, bool) & np.asarray(mask2, bool)
    l2, g2, _ = depth_mse(depth2, depth1, both)
    return l1 + l2, g1, g2


def tv_loss(components, weight=1.0):
    """TotalVariationLoss04.compute_tv_loss (src/loss_functions/TotalVariationLoss04.py:97-116)
    times ``weight``: per (1, R, H, W) component, 2 (sum of squared H differences /
    their count + the same along W), each count floored at 1 (:103-104).  Returns
    (loss, [d loss / d component])."""
    loss = 0.0
    grads = []
    for c in components:
        c = np.asarray(c)
        dt = c.dtype.type
        dh = c[:, :, 1:, :] - c[:, :, :-1, :]
        dw = c[:, :, :, 1:] - c[:, :, :, :-1]
        nh, nw = max(dh.size, 1), max(dw.size, 1)
        loss += float(weight) * 2.0 * (float(np.sum(dh * dh)) / nh + float(np.sum(dw * dw)) / nw)
        g = np.zeros_like(c)
        ch, cw = dt(4.0 * weight / nh), dt(4.0 * weight / nw)
        g[:, :, 1:, :] += ch * dh
        g[:, :, :-1, :] -= ch * dh
        g[:, :, :, 1:] += cw * dw
        g[:, :, :, :-1] -= cw * dw
        grads.append(g)
    return loss, grads


def tv_iter_weight(lr_decay_ratio, lr_decay_iters, iter_num):
    """TotalVariationLoss04.get_iter_weight (:118-120)."""
    return lr_decay_ratio ** ((iter_num + 1) / lr_decay_iters)


def coarse_fine_consistency_loss(depth_coarse, depth_fine, nerf_mask, sd_mask, rays_o, rays_d, pixel_ids, poses, k0,
                                 images, patch_size=(5, 5), rmse_threshold=0.1):
    """CoarseFineConsistencyLoss34.compute_loss (src/loss_functions/CoarseFineConsistencyLoss34.py:30-88):
    on the NeRF rays, the reprojection masks without the both-invalid rule and the
    depth term of :164-167 (as reprojection_depth_loss: mean over the NeRF rays of
    mask2 (coarse - fine)^2, gradient into the coarse depth); on the sparse-depth
    rays (compute_loss_sd, :170-187) the mean squared difference of the coarse
    depth and the detached fine depth.  Returns (loss, d/d coarse, d/d fine, mask1, mask2)."""
    nerf = np.asarray(nerf_mask, bool)
    dc, df = np.asarray(depth_coarse), np.asarray(depth_fine)
    m1, m2, _, _ = reprojection_masks(dc[nerf], df[nerf], rays_o[nerf], rays_d[nerf], pixel_ids[nerf], poses, k0,
                                      images, patch_size, rmse_threshold, both_invalid_rule=False)
    loss, g1, g2 = reprojection_depth_loss(dc[nerf], df[nerf], m1, m2)
    gc, gf = np.zeros_like(dc), np.zeros_like(df)
    gc[nerf], gf[nerf] = g1, g2
    if sd_mask is not None and np.any(sd_mask):
        sd = np.asarray(sd_mask, bool)
        l_sd, g_sd, _ = depth_mse(dc[sd], df[sd])
        loss = loss + l_sd
        gc[sd] += g_sd
    return loss, gc, gf, m1, m2
