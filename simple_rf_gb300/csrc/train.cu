// Training-step helpers: the config-2 loss gradient and a fused Adam update.
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
    for (; i < n; i += stride) {
        float gi = g[i];
        if (wd != 0.f) gi += wd * p[i];
        float mi = b1 * m[i] + (1.f - b1) * gi;
        float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        float denom = sqrtf(vi) / bc2_sqrt + eps;
        p[i] -= (lr / bc1) * mi / denom;
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

// loss += weight * mean_r m_r (pred - target)^2;  grad[r] += 2 weight m_r (pred - target) / n
__global__ void depth_consistency_kernel(const float* __restrict__ pred, const float* __restrict__ target,
                                         const uint8_t* __restrict__ mask, int n, float weight, float* loss,
                                         float* grad) {
    __shared__ float red[32];
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (r < n && (!mask || mask[r])) {
        float e = pred[r] - target[r];
        l = weight * e * e / float(n);
        grad[r] += 2.f * weight * e / float(n);
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

}  // namespace
}  // namespace srf

using namespace srf;

extern "C" int srf_depth_consistency_loss(const float* pred, const float* target, const uint8_t* mask, int n,
                                          float weight, float* loss_dev, float* grad, void* stream) {
    if (!pred || !target || !grad) return SRF_ERR_NULL;
    if (n < 0) return SRF_ERR_SHAPE;
    if (n == 0) return SRF_OK;
    depth_consistency_kernel<<<grid_1d(n, 256), 256, 0, as_stream(stream)>>>(pred, target, mask, n, weight, loss_dev,
                                                                             grad);
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
