// Training-step helpers: the training step's loss gradient and a fused Adam update.
#include "srf_common.cuh"

namespace srf {
namespace {

__global__ void loss_kernel(const float* __restrict__ rgb, const float* __restrict__ trgb,
                            const float* __restrict__ depth, const float* __restrict__ tdepth,
                            const uint8_t* __restrict__ dmask, int n, int nd, float dw, float* loss, float* g_rgb,
                            float* g_depth) {
    __shared__ float red[32];
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (r < n) {
        float inv = 2.f / float(3 * n);
        for (int c = 0; c < 3; ++c) {
            float e = rgb[3 * r + c] - trgb[3 * r + c];
            l += e * e / float(3 * n);
            g_rgb[3 * r + c] = inv * e;
        }
        float gd = 0.f;
        if (depth && dmask && dmask[r] && nd > 0) {
            float e = depth[r] - tdepth[r];
            l += dw * fabsf(e) / float(nd);
            gd = dw / float(nd) * (e > 0.f ? 1.f : (e < 0.f ? -1.f : 0.f));
        }
        if (g_depth) g_depth[r] = gd;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x < 32) {
        l = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
        if (threadIdx.x == 0 && loss) atomicAdd(loss, l);
    }
}

__device__ __forceinline__ void adam_update(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                                            float* __restrict__ v, int64_t i, float lr, float b1, float b2, float eps,
                                            float wd, float bc1, float bc2_sqrt) {
    // every rounding spelled out, so each kernel that inlines this computes the same bits
    float gi = g[i];
    if (wd != 0.f) gi = __fmaf_rn(wd, p[i], gi);
    const float mi = __fmaf_rn(b1, m[i], __fmul_rn(1.f - b1, gi));
    const float vi = __fmaf_rn(b2, v[i], __fmul_rn(__fmul_rn(1.f - b2, gi), gi));
    m[i] = mi;
    v[i] = vi;
    const float denom = __fadd_rn(__fdiv_rn(__fsqrt_rn(vi), bc2_sqrt), eps);
    p[i] = __fsub_rn(p[i], __fdiv_rn(__fmul_rn(__fdiv_rn(lr, bc1), mi), denom));
}

// torch.optim.Adam (foreach=False math): m = b1 m + (1-b1) g; v = b2 v + (1-b2) g^2;
// p -= lr / (1 - b1^t) * m / (sqrt(v) / sqrt(1 - b2^t) + eps).  With step_dev the
// step count t is read on the device (graph replays advance it with srf_counter_add).
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps, float wd,
                            float bc1, float bc2_sqrt, const int* step_dev, const int* skip_dev) {
    if (skip_dev && *skip_dev) return;
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t stride = int64_t(gridDim.x) * blockDim.x;
    if (step_dev) {
        float t = float(*step_dev);
        bc1 = 1.f - powf(b1, t);
        bc2_sqrt = sqrtf(1.f - powf(b2, t));
    }
    for (; i < n; i += stride) adam_update(p, g, m, v, i, lr, b1, b2, eps, wd, bc1, bc2_sqrt);
}

// Several tensors in one launch: tensor k covers chunks [chunk0, chunk0 + ceil(n /
// kAdamChunk)) of a common chunk index space, which the blocks stride over.
constexpr int kMaxAdamTensors = 64;
constexpr int64_t kAdamChunk = 8192;
struct AdamTensor {
    float* p;
    const float* g;
    float* m;
    float* v;
    int64_t n;
    float lr;
    int64_t chunk0;
};
struct AdamBatch {
    AdamTensor t[kMaxAdamTensors];
    int count;
    int64_t chunks;
};

__global__ void adam_multi_kernel(const __grid_constant__ AdamBatch b, float b1, float b2, float eps, float wd,
                                  float bc1, float bc2_sqrt, const int* step_dev, const int* skip_dev) {
    if (skip_dev && *skip_dev) return;
    if (step_dev) {
        float t = float(*step_dev);
        bc1 = 1.f - powf(b1, t);
        bc2_sqrt = sqrtf(1.f - powf(b2, t));
    }
    int k = 0;
    for (int64_t ch = blockIdx.x; ch < b.chunks; ch += gridDim.x) {
        while (k + 1 < b.count && b.t[k + 1].chunk0 <= ch) ++k;
        const AdamTensor& t = b.t[k];
        const int64_t i0 = (ch - t.chunk0) * kAdamChunk;
        const int64_t i1 = i0 + kAdamChunk < t.n ? i0 + kAdamChunk : t.n;
        for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x)
            adam_update(t.p, t.g, t.m, t.v, i, t.lr, b1, b2, eps, wd, bc1, bc2_sqrt);
    }
}

__global__ void counter_add_kernel(int* c, int v, const int* skip) {
    if (!skip || !*skip) *c += v;
}

__global__ void loss_scaler_init_kernel(srf_loss_scaler* s, float init) {
    s->scale = init;
    s->inv_scale = 1.f / init;
    s->found_inf = 0;
    s->growth_tracker = 0;
}

// growth_tracker (as float bits) <- max |x| over a and b (non-negative floats order like their bits).
__global__ void absmax_kernel(const float* __restrict__ a, int64_t na, const float* __restrict__ b, int64_t nb,
                              srf_loss_scaler* s) {
    float mx = 0.f;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < na + nb; i += stride) {
        float v = fabsf(i < na ? a[i] : b[i - na]);
        mx = v > mx ? v : mx;   // a NaN never wins, so a non-finite input leaves the scale finite
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(&s->growth_tracker, __float_as_int(mx));
}

// scale = 2^floor(log2(target / max)), within [2^-24, 2^40]; 1 when max is 0 or not finite.
__global__ void fit_scale_kernel(srf_loss_scaler* s, float target) {
    float mx = __int_as_float(s->growth_tracker);
    float sc = 1.f;
    if (mx > 0.f && mx < 3.0e38f) {
        int e = int(floorf(log2f(target / mx)));
        e = e < -24 ? -24 : (e > 40 ? 40 : e);
        sc = ldexpf(1.f, e);
    }
    s->scale = sc;
    s->inv_scale = 1.f / sc;
    s->found_inf = 0;
    s->growth_tracker = 0;
}

__global__ void loss_scaler_update_kernel(srf_loss_scaler* s, float growth, float backoff, int interval) {
    if (s->found_inf) {
        s->scale *= backoff;
        s->growth_tracker = 0;
    } else if (++s->growth_tracker >= interval) {
        s->scale *= growth;
        s->growth_tracker = 0;
    }
    s->inv_scale = 1.f / s->scale;
    s->found_inf = 0;
}

// Block-wide sum over the 1024 threads of one block (callable by every thread).
template <class T>
__device__ T block_sum(T v, T* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : T(0);
    if (threadIdx.x < 32) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    if (threadIdx.x == 0) red[0] = v;
    __syncthreads();
    v = red[0];
    __syncthreads();
    return v;
}

// Number of rays the mean runs over: the masked ones, or all n.
__device__ int mean_count(const uint8_t* mask, int n, int over_mask, int* ired) {
    if (!over_mask || !mask) return n;
    int c = 0;
    for (int r = threadIdx.x; r < n; r += blockDim.x) c += mask[r] != 0;
    return block_sum(c, ired);
}

// loss += weight * sum_r m_r (pred - target)^2 / count and the matching gradients
// (one block of 1024 threads: the count precedes every term).
__global__ void depth_mse_kernel(const float* __restrict__ pred, const float* __restrict__ target,
                                 const uint8_t* __restrict__ mask, int n, float weight, int over_mask, float* loss,
                                 float* gp, float* gt) {
    __shared__ float fred[32];
    __shared__ int ired[32];
    const int cnt = mean_count(mask, n, over_mask, ired);
    if (cnt == 0) return;
    const float inv = 1.f / float(cnt);
    float l = 0.f;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        if (mask && !mask[r]) continue;
        const float e = pred[r] - target[r];
        l += e * e;
        const float g = weight * 2.f * e * inv;
        if (gp) gp[r] += g;
        if (gt) gt[r] -= g;
    }
    l = block_sum(l, fred);
    if (threadIdx.x == 0 && loss) atomicAdd(loss, weight * l * inv);
}

// Per ray: bin sums b_k of the weights, loss term -sum_k (b_k + 1e-3) ln(b_k + 1e-3);
// mean over the (masked) rays; d/dw_i = -(ln(b_k + 1e-3) + 1) for i in bin k.  One
// block of 1024 threads, a warp per ray and a lane per bin.
__global__ void mass_concentration_kernel(const float* __restrict__ w, int n, int s, BinLayout bl,
                                          const uint8_t* __restrict__ mask, float weight, float* loss, float* gw) {
    __shared__ float fred[32];
    __shared__ int ired[32];
    const int cnt = mean_count(mask, n, 1, ired);
    if (cnt == 0) return;
    const float scale = weight / float(cnt);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    float l = 0.f;
    for (int r = warp; r < n; r += nw) {
        if (mask && !mask[r]) continue;
        const float* wr = w + int64_t(r) * s;
        for (int b = lane; b < bl.nb; b += 32) {
            float sum = 0.f;
            for (int i = bl.start[b]; i < bl.start[b + 1]; ++i) sum += wr[i];
            const float x = sum + 1e-3f;
            const float lx = logf(x);
            l -= x * lx;
            if (gw) {
                const float g = -(lx + 1.f) * scale;
                float* gr = gw + int64_t(r) * s;
                for (int i = bl.start[b]; i < bl.start[b + 1]; ++i) gr[i] += g;
            }
        }
    }
    l = block_sum(l, fred);
    if (threadIdx.x == 0 && loss) atomicAdd(loss, l * scale);
}

// AugmentationsDepthLoss11.compute_loss_nerf masks (AugmentationsDepthLoss11.py:105-190),
// one thread per ray: the nearest other camera b, both depths' points reprojected
// into b (CommonUtils04.reproject: ((K0 diag(1,-1,-1)) R_b^T) (p - t_b), then x/z,
// y/z, rounded half to even), the RMSE of the ray's patch in its own image against
// the patch at each reprojection in image b (zero outside the image), and the
// reference's mask rules.
// a0 b0 + a1 b1 + a2 b2 with each product and sum rounded separately (no FMA),
// as the reference's small float32 matrix products round
__device__ __forceinline__ float dot3_rn(float a0, float a1, float a2, float b0, float b1, float b2) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a0, b0), __fmul_rn(a1, b1)), __fmul_rn(a2, b2));
}

__device__ __forceinline__ float patch_rmse(const float* __restrict__ imgs, int H, int W, int C, int ia, int ya,
                                            int xa, int ib, int yb, int xb, int hpy, int hpx) {
    float acc = 0.f;
    for (int dy = -hpy; dy <= hpy; ++dy) {
        for (int dx = -hpx; dx <= hpx; ++dx) {
            const int y1 = ya + dy, x1 = xa + dx, y2 = yb + dy, x2 = xb + dx;
            const bool in1 = y1 >= 0 && y1 < H && x1 >= 0 && x1 < W;
            const bool in2 = y2 >= 0 && y2 < H && x2 >= 0 && x2 < W;
            const float* p1 = in1 ? imgs + ((int64_t(ia) * H + y1) * W + x1) * C : nullptr;
            const float* p2 = in2 ? imgs + ((int64_t(ib) * H + y2) * W + x2) * C : nullptr;
            for (int c = 0; c < C; ++c) {
                const float e = (p1 ? p1[c] : 0.f) - (p2 ? p2[c] : 0.f);
                acc += e * e;
            }
        }
    }
    return sqrtf(acc / float((2 * hpy + 1) * (2 * hpx + 1) * C));
}

__global__ void reprojection_masks_kernel(const float* __restrict__ ro, const float* __restrict__ rd,
                                          const float* __restrict__ d1, const float* __restrict__ d2,
                                          const int32_t* __restrict__ pid, int n, const float* __restrict__ poses,
                                          int V, const float* __restrict__ k0, const float* __restrict__ imgs, int H,
                                          int W, int C, int hpx, int hpy, float thr, int both_invalid_rule,
                                          uint8_t* m1, uint8_t* m2, int* flag) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int ia = pid[3 * r], xa = pid[3 * r + 1], ya = pid[3 * r + 2];
    if (ia < 0 || ia >= V) {
        m1[r] = m2[r] = 0;
        raise_flag(flag, kFlagRange);
        return;
    }
    // nearest other camera origin (ties: lowest index)
    const float* pa = poses + 16 * ia;
    int ib = -1;
    float best = 0.f;
    for (int j = 0; j < V; ++j) {
        if (j == ia) continue;
        const float* pj = poses + 16 * j;
        const float ex = pa[3] - pj[3], ey = pa[7] - pj[7], ez = pa[11] - pj[11];
        const float dist = sqrtf(ex * ex + ey * ey + ez * ez);
        if (ib < 0 || dist < best) {
            ib = j;
            best = dist;
        }
    }
    if (ib < 0) {   // a single view: nothing to compare against
        m1[r] = m2[r] = 0;
        return;
    }
    const float* pb = poses + 16 * ib;
    // M = (K0 diag(1, -1, -1)) R_b^T, row by row
    float kp[9];
    for (int i = 0; i < 3; ++i) {
        kp[3 * i] = k0[3 * i];
        kp[3 * i + 1] = -k0[3 * i + 1];
        kp[3 * i + 2] = -k0[3 * i + 2];
    }
    float M[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)   // (R^T)[k][j] = R[j][k]
            M[3 * i + j] = dot3_rn(kp[3 * i], kp[3 * i + 1], kp[3 * i + 2], pb[4 * j], pb[4 * j + 1], pb[4 * j + 2]);
    int qx[2], qy[2];
    for (int s = 0; s < 2; ++s) {
        const float dep = s == 0 ? d1[r] : d2[r];
        float v[3];
        for (int a = 0; a < 3; ++a)
            v[a] = __fsub_rn(__fadd_rn(ro[3 * r + a], __fmul_rn(rd[3 * r + a], dep)), pb[4 * a + 3]);
        float p[3];
        for (int i = 0; i < 3; ++i) p[i] = dot3_rn(M[3 * i], M[3 * i + 1], M[3 * i + 2], v[0], v[1], v[2]);
        const float fx = rintf(p[0] / p[2]), fy = rintf(p[1] / p[2]);
        // far-off or non-finite positions: any out-of-image value keeps the masks' logic
        qx[s] = isfinite(fx) ? int(fminf(fmaxf(fx, -1e6f), 1e6f)) : -1000000;
        qy[s] = isfinite(fy) ? int(fminf(fmaxf(fy, -1e6f), 1e6f)) : -1000000;
    }
    auto valid = [&](int x, int y) { return x >= hpx && x < W - hpx && y >= hpy && y < H - hpy; };
    const bool va = valid(xa, ya), v1 = valid(qx[0], qy[0]), v2 = valid(qx[1], qy[1]);
    const int cx1 = min(max(qx[0], 0), W - 1), cy1 = min(max(qy[0], 0), H - 1);
    const int cx2 = min(max(qx[1], 0), W - 1), cy2 = min(max(qy[1], 0), H - 1);
    const int xs = min(max(xa, 0), W - 1), ys = min(max(ya, 0), H - 1);
    const float r1 = patch_rmse(imgs, H, W, C, ia, ys, xs, ib, cy1, cx1, hpy, hpx);
    const float r2 = patch_rmse(imgs, H, W, C, ia, ys, xs, ib, cy2, cx2, hpy, hpx);
    bool a = ((r1 < r2) || !v2) && (r1 < thr) && v1 && va;
    bool b = ((r2 < r1) || !v1) && (r2 < thr) && v2 && va;
    if (both_invalid_rule && !(v1 || v2)) {
        a = a || (d1[r] > d2[r]);
        b = b || (d2[r] > d1[r]);
    }
    m1[r] = a;
    m2[r] = b;
}

// pts[r * S + i] = o[r] + d[r] * z[r, i]  (SimpleNeRF17.py:213-215).  The product
// and the sum round separately, as the reference's two torch ops do: PE scales
// pts by up to 2^9, so a one-ulp difference here moves the network's output.
__global__ void ray_points_kernel(const float* __restrict__ o, const float* __restrict__ d,
                                  const float* __restrict__ z, int64_t n, int s, float* pts) {
    int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= n * s) return;
    int64_t r = idx / s;
    float zz = z[idx];
#pragma unroll
    for (int a = 0; a < 3; ++a) pts[3 * idx + a] = __fadd_rn(o[3 * r + a], __fmul_rn(d[3 * r + a], zz));
}

// One component of the total-variation loss: an (R, H, W) grid with element
// strides (sr, sh, sw), its gradient (same strides) and the loss weights of the
// H and W differences, weight * 2 / numel.
struct TvComp {
    const float* p;
    float* g;
    int r, h, w;
    int64_t sr, sh, sw;
    float ch, cw;
};
constexpr int kMaxTvComps = 8;
struct TvBatch {
    TvComp c[kMaxTvComps];
};

// TotalVariationLoss04.compute_tv_loss (TotalVariationLoss04.py:97-116):
// loss += sum ch (P[h+1] - P[h])^2 + cw (P[w+1] - P[w])^2 over the component,
// grad += scale * d loss / dP, a thread per element (r fastest, so a channels-last
// grid is read in order).  blockIdx.y picks the component.
__global__ void __launch_bounds__(256) tv_kernel(const __grid_constant__ TvBatch b, const float* scale_dev,
                                                 float* loss) {
    __shared__ float red[32];
    const TvComp& c = b.c[blockIdx.y];
    const float gs = scale_dev ? *scale_dev : 1.f;
    const uint32_t n = uint32_t(c.r) * uint32_t(c.h) * uint32_t(c.w);
    float l = 0.f;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t r = j % uint32_t(c.r), t = j / uint32_t(c.r);
        const int w = int(t % uint32_t(c.w)), h = int(t / uint32_t(c.w));
        const int64_t off = int64_t(r) * c.sr + int64_t(h) * c.sh + int64_t(w) * c.sw;
        const float x = c.p[off];
        const float dn = h + 1 < c.h ? c.p[off + c.sh] - x : 0.f;    // P[h+1] - P[h]
        const float up = h > 0 ? x - c.p[off - c.sh] : 0.f;          // P[h] - P[h-1]
        const float rt = w + 1 < c.w ? c.p[off + c.sw] - x : 0.f;
        const float lf = w > 0 ? x - c.p[off - c.sw] : 0.f;
        l += c.ch * dn * dn + c.cw * rt * rt;
        if (c.g) c.g[off] += gs * 2.f * (c.ch * (up - dn) + c.cw * (lf - rt));
    }
    l = block_sum(l, red);
    if (loss && threadIdx.x == 0 && l != 0.f) atomicAdd(loss, l);
}

}  // namespace
}  // namespace srf

using namespace srf;

extern "C" int srf_depth_mse_loss(const float* pred, const float* target, const uint8_t* mask, int n, float weight,
                                  int mean_over_mask, float* loss_dev, float* grad_pred, float* grad_target,
                                  void* stream) {
    if (n < 0) return SRF_ERR_SHAPE;
    if (n == 0) return SRF_OK;
    if (!pred || !target) return SRF_ERR_NULL;
    depth_mse_kernel<<<1, 1024, 0, as_stream(stream)>>>(pred, target, mask, n, weight, mean_over_mask, loss_dev,
                                                        grad_pred, grad_target);
    return launch_status();
}

extern "C" int srf_mass_concentration_loss(const float* weights, int n_rays, int n_samples, int num_bins,
                                           const uint8_t* mask, float weight, float* loss_dev, float* grad_weights,
                                           void* stream) {
    if (n_rays < 0) return SRF_ERR_SHAPE;
    BinLayout bl;
    if (!bin_layout(n_samples, num_bins, &bl)) return SRF_ERR_SHAPE;
    if (n_rays == 0) return SRF_OK;
    if (!weights) return SRF_ERR_NULL;
    mass_concentration_kernel<<<1, 1024, 0, as_stream(stream)>>>(weights, n_rays, n_samples, bl, mask, weight,
                                                                 loss_dev, grad_weights);
    return launch_status();
}

extern "C" int srf_counter_add(int32_t* counter_dev, int value, const int32_t* skip_dev, void* stream) {
    if (!counter_dev) return SRF_ERR_NULL;
    counter_add_kernel<<<1, 1, 0, as_stream(stream)>>>(counter_dev, value, skip_dev);
    return launch_status();
}

extern "C" int srf_loss_scaler_init(srf_loss_scaler* scaler_dev, float init_scale, void* stream) {
    if (!scaler_dev) return SRF_ERR_NULL;
    if (!(init_scale > 0.f)) return SRF_ERR_SHAPE;
    loss_scaler_init_kernel<<<1, 1, 0, as_stream(stream)>>>(scaler_dev, init_scale);
    return launch_status();
}

extern "C" int srf_loss_scaler_fit(srf_loss_scaler* scaler_dev, const float* a, int64_t na, const float* b,
                                   int64_t nb, float target, void* stream) {
    if (!scaler_dev || (na > 0 && !a) || (nb > 0 && !b)) return SRF_ERR_NULL;
    if (na < 0 || nb < 0 || !(target > 0.f)) return SRF_ERR_SHAPE;
    cudaStream_t st = as_stream(stream);
    cudaError_t e = cudaMemsetAsync(&scaler_dev->growth_tracker, 0, sizeof(int32_t), st);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return SRF_ERR_CUDA;
    }
    if (na + nb > 0) {
        unsigned blocks = grid_1d(na + nb, 256);
        if (blocks > 152 * 4) blocks = 152 * 4;
        absmax_kernel<<<blocks, 256, 0, st>>>(a, na, b, nb, scaler_dev);
        int ls = launch_status();
        if (ls) return ls;
    }
    fit_scale_kernel<<<1, 1, 0, st>>>(scaler_dev, target);
    return launch_status();
}

extern "C" int srf_loss_scaler_update(srf_loss_scaler* scaler_dev, float growth, float backoff, int growth_interval,
                                      void* stream) {
    if (!scaler_dev) return SRF_ERR_NULL;
    if (!(growth >= 1.f) || !(backoff > 0.f) || !(backoff <= 1.f) || growth_interval < 1) return SRF_ERR_SHAPE;
    loss_scaler_update_kernel<<<1, 1, 0, as_stream(stream)>>>(scaler_dev, growth, backoff, growth_interval);
    return launch_status();
}

extern "C" int srf_ray_points(const float* rays_o, const float* rays_d, const float* z, int n_rays, int n_samples,
                              float* pts, void* stream) {
    if (!rays_o || !rays_d || !z || !pts) return SRF_ERR_NULL;
    if (n_rays < 0 || n_samples < 1) return SRF_ERR_SHAPE;
    if (n_rays == 0) return SRF_OK;
    int64_t tot = int64_t(n_rays) * n_samples;
    ray_points_kernel<<<grid_1d(tot, 256), 256, 0, as_stream(stream)>>>(rays_o, rays_d, z, n_rays, n_samples, pts);
    return launch_status();
}

extern "C" int srf_rgb_depth_loss(const float* rgb, const float* target_rgb, const float* depth,
                                  const float* target_depth, const uint8_t* depth_mask, int n_rays, int n_depth_rays,
                                  float depth_weight, float* loss_dev, float* g_rgb, float* g_depth, void* stream) {
    if (!rgb || !target_rgb || !g_rgb) return SRF_ERR_NULL;
    if (depth_mask && (!depth || !target_depth)) return SRF_ERR_NULL;
    if (n_rays < 0 || n_depth_rays < 0) return SRF_ERR_SHAPE;
    if (n_rays == 0) return SRF_OK;
    loss_kernel<<<grid_1d(n_rays, 256), 256, 0, as_stream(stream)>>>(rgb, target_rgb, depth, target_depth, depth_mask,
                                                                     n_rays, n_depth_rays, depth_weight, loss_dev,
                                                                     g_rgb, g_depth);
    return launch_status();
}

extern "C" int srf_adam_step(float* param, const float* grad, float* exp_avg, float* exp_avg_sq, int64_t n, float lr,
                             float beta1, float beta2, float eps, float weight_decay, int step,
                             const int32_t* step_dev, const int32_t* skip_dev, void* stream) {
    if (!param || !grad || !exp_avg || !exp_avg_sq) return SRF_ERR_NULL;
    if (n < 0 || (step < 1 && !step_dev)) return SRF_ERR_SHAPE;
    if (step < 1) step = 1;
    if (n == 0) return SRF_OK;
    float bc1 = 1.f - powf(beta1, float(step));
    float bc2 = sqrtf(1.f - powf(beta2, float(step)));
    unsigned blocks = grid_1d(n, 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    adam_kernel<<<blocks, 256, 0, as_stream(stream)>>>(param, grad, exp_avg, exp_avg_sq, n, lr, beta1, beta2, eps,
                                                       weight_decay, bc1, bc2, step_dev, skip_dev);
    return launch_status();
}

extern "C" int srf_adam_multi_step(const srf_adam_tensor* tensors, int n_tensors, float beta1, float beta2, float eps,
                                   float weight_decay, int step, const int32_t* step_dev, const int32_t* skip_dev,
                                   void* stream) {
    if (n_tensors < 0 || (step < 1 && !step_dev)) return SRF_ERR_SHAPE;
    if (n_tensors == 0) return SRF_OK;
    if (!tensors) return SRF_ERR_NULL;
    for (int i = 0; i < n_tensors; ++i) {
        const srf_adam_tensor& t = tensors[i];
        if (t.n < 0) return SRF_ERR_SHAPE;
        if (t.n > 0 && (!t.param || !t.grad || !t.exp_avg || !t.exp_avg_sq)) return SRF_ERR_NULL;
    }
    if (step < 1) step = 1;
    const float bc1 = 1.f - powf(beta1, float(step));
    const float bc2 = sqrtf(1.f - powf(beta2, float(step)));
    int i = 0;   // next tensor: each launch takes up to kMaxAdamTensors non-empty ones
    while (i < n_tensors) {
        AdamBatch b = {};
        int64_t chunks = 0;
        for (; i < n_tensors && b.count < kMaxAdamTensors; ++i) {
            const srf_adam_tensor& t = tensors[i];
            if (t.n == 0) continue;
            b.t[b.count++] = {t.param, t.grad, t.exp_avg, t.exp_avg_sq, t.n, t.lr, chunks};
            chunks += (t.n + kAdamChunk - 1) / kAdamChunk;
        }
        if (!chunks) continue;
        b.chunks = chunks;
        unsigned blocks = unsigned(chunks < 152 * 8 ? chunks : 152 * 8);
        adam_multi_kernel<<<blocks, 256, 0, as_stream(stream)>>>(b, beta1, beta2, eps, weight_decay, bc1, bc2,
                                                                 step_dev, skip_dev);
        int st = launch_status();
        if (st) return st;
    }
    return SRF_OK;
}

static int reprojection_masks(const float* rays_o, const float* rays_d, const float* depth1, const float* depth2,
                              const int32_t* pixel_ids, int n_rays, const float* poses, int n_views,
                              const float* intrinsics0, const float* images, int height, int width, int channels,
                              int patch_w, int patch_h, float rmse_threshold, int both_invalid_rule, uint8_t* mask1,
                              uint8_t* mask2, void* stream) {
    if (n_rays < 0 || n_views < 1 || height < 1 || width < 1 || channels < 1 || channels > 64) return SRF_ERR_SHAPE;
    if (patch_w < 1 || patch_h < 1 || patch_w > 31 || patch_h > 31) return SRF_ERR_SHAPE;
    if (n_rays == 0) return SRF_OK;
    if (!rays_o || !rays_d || !depth1 || !depth2 || !pixel_ids || !poses || !intrinsics0 || !images || !mask1 ||
        !mask2)
        return SRF_ERR_NULL;
    reprojection_masks_kernel<<<grid_1d(n_rays, 128), 128, 0, as_stream(stream)>>>(
        rays_o, rays_d, depth1, depth2, pixel_ids, n_rays, poses, n_views, intrinsics0, images, height, width,
        channels, patch_w / 2, patch_h / 2, rmse_threshold, both_invalid_rule, mask1, mask2, device_flag());
    return launch_status();
}

extern "C" int srf_depth_reprojection_masks(const float* rays_o, const float* rays_d, const float* depth1,
                                            const float* depth2, const int32_t* pixel_ids, int n_rays,
                                            const float* poses, int n_views, const float* intrinsics0,
                                            const float* images, int height, int width, int channels, int patch_w,
                                            int patch_h, float rmse_threshold, uint8_t* mask1, uint8_t* mask2,
                                            void* stream) {
    return reprojection_masks(rays_o, rays_d, depth1, depth2, pixel_ids, n_rays, poses, n_views, intrinsics0, images,
                              height, width, channels, patch_w, patch_h, rmse_threshold, 1, mask1, mask2, stream);
}

extern "C" int srf_coarse_fine_reprojection_masks(const float* rays_o, const float* rays_d, const float* depth_coarse,
                                                  const float* depth_fine, const int32_t* pixel_ids, int n_rays,
                                                  const float* poses, int n_views, const float* intrinsics0,
                                                  const float* images, int height, int width, int channels,
                                                  int patch_w, int patch_h, float rmse_threshold, uint8_t* mask1,
                                                  uint8_t* mask2, void* stream) {
    return reprojection_masks(rays_o, rays_d, depth_coarse, depth_fine, pixel_ids, n_rays, poses, n_views,
                              intrinsics0, images, height, width, channels, patch_w, patch_h, rmse_threshold, 0, mask1,
                              mask2, stream);
}

extern "C" int srf_tv_loss(const srf_tv_component* components, int n_components, float weight, const float* scale_dev,
                           float* loss_dev, void* stream) {
    if (n_components < 0 || n_components > kMaxTvComps) return SRF_ERR_SHAPE;
    if (n_components == 0) return SRF_OK;
    if (!components) return SRF_ERR_NULL;
    TvBatch b = {};
    uint32_t most = 0;
    for (int i = 0; i < n_components; ++i) {
        const srf_tv_component& s = components[i];
        if (s.channels < 1 || s.height < 1 || s.width < 1) return SRF_ERR_SHAPE;
        const int64_t n = int64_t(s.channels) * s.height * s.width;
        if (n > int64_t(0x7fffffff)) return SRF_ERR_SHAPE;
        if (!s.data) return SRF_ERR_NULL;
        // numel of the difference tensors, at least 1 (TotalVariationLoss04.py:103-104)
        const int64_t nh = int64_t(s.channels) * (s.height - 1) * s.width;
        const int64_t nw = int64_t(s.channels) * s.height * (s.width - 1);
        b.c[i] = {s.data, s.grad, s.channels, s.height, s.width, s.stride_channel, s.stride_height, s.stride_width,
                  float(2.0 * weight / double(nh > 1 ? nh : 1)), float(2.0 * weight / double(nw > 1 ? nw : 1))};
        if (uint32_t(n) > most) most = uint32_t(n);
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    unsigned gx = grid_1d(most, 256);
    const unsigned cap = unsigned(sms > 0 ? sms : 152) * 8u / unsigned(n_components);
    if (gx > cap) gx = cap > 0 ? cap : 1;
    tv_kernel<<<dim3(gx, n_components), 256, 0, as_stream(stream)>>>(b, scale_dev, loss_dev);
    return launch_status();
}
