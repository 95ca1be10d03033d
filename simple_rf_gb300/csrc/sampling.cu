// Ray generation and sampling kernels.  Compiled with -fmad=false so each
// formula rounds like the reference's sequence of separate torch ops.
#include "srf_common.cuh"

namespace srf {
namespace {

// torch.linspace(start, end, steps)[i], the scalar (CUDA) formula: the first
// half counts up from start, the second half counts down from end.
__device__ __forceinline__ float linspace_at(float start, float end, int steps, int i) {
    if (steps == 1) return start;
    float step = (end - start) / float(steps - 1);
    int half = steps / 2;
    return i < half ? start + step * float(i) : end - step * float(steps - i - 1);
}

__global__ void ndc_rays_kernel(const float* __restrict__ o, const float* __restrict__ d, const float* fx,
                                const float* fy, int n, float h, float w, float near_plane, float* o_ndc,
                                float* d_ndc, float* vdirs) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    float dx = d[3 * r], dy = d[3 * r + 1], dz = d[3 * r + 2];
    if (vdirs) {
        float nrm = sqrtf(dx * dx + dy * dy + dz * dz);
        vdirs[3 * r] = dx / nrm;
        vdirs[3 * r + 1] = dy / nrm;
        vdirs[3 * r + 2] = dz / nrm;
    }
    if (!o_ndc && !d_ndc) return;
    // only reached when the host checked that o, fx and fy are non-NULL
    float ox = o[3 * r], oy = o[3 * r + 1], oz = o[3 * r + 2];
    // CommonUtils04.py:124-137
    float t = -(near_plane + oz) / dz;
    float sx = ox + t * dx, sy = oy + t * dy, sz = oz + t * dz;
    float ax = -1.f / (w / (2.f * fx[r]));
    float ay = -1.f / (h / (2.f * fy[r]));
    if (o_ndc) {
        o_ndc[3 * r] = ax * sx / sz;
        o_ndc[3 * r + 1] = ay * sy / sz;
        o_ndc[3 * r + 2] = 1.f + 2.f * near_plane / sz;
    }
    if (d_ndc) {
        d_ndc[3 * r] = ax * (dx / dz - sx / sz);
        d_ndc[3 * r + 1] = ay * (dy / dz - sy / sz);
        d_ndc[3 * r + 2] = -2.f * near_plane / sz;
    }
}

// CommonUtils04.py:73-95 get_rays_tr (non-synthetic branch): dirs = K^-1 [x, y, 1]
// (y and z negated), rotated by the camera-to-world matrix; origin = its translation.
// K^-1 by the adjugate (K is a 3x3 intrinsics matrix).
__global__ void pixel_rays_kernel(const int* __restrict__ pix, const float* __restrict__ K,
                                  const float* __restrict__ E, int n, int half_pixel, float* o, float* d) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    float x = float(pix[3 * r + 1]), y = float(pix[3 * r + 2]);
    if (half_pixel) {
        x = x + 0.5f;
        y = y + 0.5f;
    }
    const float* k = K + 9 * r;
    float a = k[0], b = k[1], c = k[2], dd = k[3], e = k[4], f = k[5], g = k[6], h = k[7], i = k[8];
    float A = e * i - f * h, B = -(dd * i - f * g), C = dd * h - e * g;
    float det = a * A + b * B + c * C;
    float inv[9] = {A / det, -(b * i - c * h) / det, (b * f - c * e) / det,
                    B / det, (a * i - c * g) / det, -(a * f - c * dd) / det,
                    C / det, -(a * h - b * g) / det, (a * e - b * dd) / det};
    float cam[3];
    for (int q = 0; q < 3; ++q) cam[q] = inv[3 * q] * x + inv[3 * q + 1] * y + inv[3 * q + 2];
    cam[1] = -cam[1];
    cam[2] = -cam[2];
    const float* m = E + 16 * r;
    for (int q = 0; q < 3; ++q) {
        d[3 * r + q] = cam[0] * m[4 * q] + cam[1] * m[4 * q + 1] + cam[2] * m[4 * q + 2];
        o[3 * r + q] = m[4 * q + 3];
    }
}

__device__ __forceinline__ float base_z(float near_plane, float far_plane, int s, int i, int lindisp) {
    float t = linspace_at(0.f, 1.f, s, i);
    if (!lindisp) return near_plane * (1.f - t) + far_plane * t;
    return 1.f / (1.f / near_plane * (1.f - t) + 1.f / far_plane * t);
}

__global__ void stratified_kernel(float* z, const float* u, int n, int s, float near_plane, float far_plane,
                                  int lindisp) {
    int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= int64_t(n) * s) return;
    int i = int(idx % s);
    float zi = base_z(near_plane, far_plane, s, i, lindisp);
    if (u) {
        // SimpleNeRF17.py:351-357
        float lower = zi, upper = zi;
        if (i > 0) lower = .5f * (zi + base_z(near_plane, far_plane, s, i - 1, lindisp));
        if (i < s - 1) upper = .5f * (base_z(near_plane, far_plane, s, i + 1, lindisp) + zi);
        zi = lower + (upper - lower) * u[idx];
    }
    z[idx] = zi;
}

// Inclusive warp scan (Hillis-Steele) of one value per lane.
__device__ __forceinline__ float warp_inclusive_sum(float v) {
    unsigned lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        float t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= unsigned(o)) v += t;
    }
    return v;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Builds the cdf (n_w + 1 entries, cdf[0] = 0) of weights + 1e-5 in shared memory.
// One warp; chunked inclusive scan.  SimpleNeRF17.py:387-390.
__device__ void build_cdf(const float* __restrict__ w, int n_w, float* cdf) {
    unsigned lane = threadIdx.x & 31;
    float part = 0.f;
    for (int j = lane; j < n_w; j += 32) part += w[j] + 1e-5f;
    float total = warp_sum(part);
    float carry = 0.f;
    if (lane == 0) cdf[0] = 0.f;
    for (int base = 0; base < n_w; base += 32) {
        int j = base + lane;
        float p = j < n_w ? (w[j] + 1e-5f) / total : 0.f;
        float inc = warp_inclusive_sum(p) + carry;
        if (j < n_w) cdf[j + 1] = inc;
        carry = __shfl_sync(0xffffffffu, inc, 31);
    }
    __syncwarp();
}

// One inverse-CDF sample: searchsorted(right=True), clamp, gather, lerp.  :401-415
__device__ __forceinline__ float invert_cdf(const float* cdf, const float* bins, int n_cdf, float u) {
    int lo = 0, hi = n_cdf;   // first index with cdf[idx] > u
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (cdf[mid] <= u) lo = mid + 1; else hi = mid;
    }
    int below = lo - 1 < 0 ? 0 : lo - 1;
    int above = lo > n_cdf - 1 ? n_cdf - 1 : lo;
    float c0 = cdf[below], c1 = cdf[above];
    float b0 = bins[below], b1 = bins[above];
    float denom = c1 - c0;
    if (denom < 1e-5f) denom = 1.f;
    float t = (u - c0) / denom;
    return b0 + t * (b1 - b0);
}

// One warp per ray.  Shared memory per warp: cdf[n_bins] + bins[n_bins].
__global__ void sample_pdf_kernel(float* samples, const float* __restrict__ bins, const float* __restrict__ weights,
                                  const float* __restrict__ u, int n, int n_bins, int n_samples) {
    extern __shared__ float smem[];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int ray = blockIdx.x * (blockDim.x >> 5) + warp;
    if (ray >= n) return;
    float* cdf = smem + warp * 2 * n_bins;
    float* sb = cdf + n_bins;
    for (int j = lane; j < n_bins; j += 32) sb[j] = bins[int64_t(ray) * n_bins + j];
    build_cdf(weights + int64_t(ray) * (n_bins - 1), n_bins - 1, cdf);
    for (int j = lane; j < n_samples; j += 32) {
        float uu = u ? u[int64_t(ray) * n_samples + j] : linspace_at(0.f, 1.f, n_samples, j);
        samples[int64_t(ray) * n_samples + j] = invert_cdf(cdf, sb, n_bins, uu);
    }
}

// One warp per ray: mids of z_coarse, pdf samples from weights[1:-1], then a
// rank-based merge sort of [z_coarse, samples] (SimpleNeRF17.py:366-370).
// Shared memory per warp: cdf[nc-1] + mids[nc-1] + vals[nc+nf].
__global__ void fine_z_kernel(float* z_fine, const float* __restrict__ zc, const float* __restrict__ wc,
                              const float* __restrict__ u, int n, int nc, int nf) {
    extern __shared__ float smem[];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int ray = blockIdx.x * (blockDim.x >> 5) + warp;
    if (ray >= n) return;
    int nb = nc - 1, tot = nc + nf;
    float* cdf = smem + warp * (2 * nb + tot);
    float* mids = cdf + nb;
    float* vals = mids + nb;
    const float* z = zc + int64_t(ray) * nc;
    for (int j = lane; j < nc; j += 32) {
        float zj = z[j];
        vals[j] = zj;
        if (j < nb) mids[j] = .5f * (z[j + 1] + zj);
    }
    build_cdf(wc + int64_t(ray) * nc + 1, nb - 1, cdf);
    __syncwarp();
    for (int j = lane; j < nf; j += 32) {
        float uu = u ? u[int64_t(ray) * nf + j] : linspace_at(0.f, 1.f, nf, j);
        vals[nc + j] = invert_cdf(cdf, mids, nb, uu);
    }
    __syncwarp();
    float* out = z_fine + int64_t(ray) * tot;
    for (int j = lane; j < tot; j += 32) {
        float v = vals[j];
        int rank = 0;
        for (int k = 0; k < tot; ++k) {
            float w = vals[k];
            rank += (w < v) || (w == v && k < j);
        }
        out[rank] = v;
    }
}

__global__ void aabb_z_kernel(float* z, const float* __restrict__ o, const float* __restrict__ d,
                              const float* __restrict__ u, int n, int s, float b0x, float b0y, float b0z,
                              float b1x, float b1y, float b1z, float near_plane, float far_plane, float step) {
    int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= int64_t(n) * s) return;
    int r = int(idx / s), i = int(idx % s);
    const float b0[3] = {b0x, b0y, b0z}, b1[3] = {b1x, b1y, b1z};
    float tmin = -INFINITY;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float dv = d[3 * r + a];
        float vec = dv == 0.f ? 1e-6f : dv;
        float ra = (b1[a] - o[3 * r + a]) / vec;
        float rb = (b0[a] - o[3 * r + a]) / vec;
        float mn = fminf(ra, rb);
        tmin = fmaxf(tmin, mn);
    }
    tmin = fminf(fmaxf(tmin, near_plane), far_plane);
    float rng = float(i);
    if (u) rng = rng + u[r];
    z[idx] = tmin + step * rng;
}

__global__ void pe_kernel(float* out, int ld, const float* __restrict__ x, int64_t m, int dims, int degree) {
    int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= m * dims) return;
    int64_t row = idx / dims;
    int j = int(idx % dims);
    float v = x[idx];
    float* o = out + row * ld;
    o[j] = v;
    float f = 1.f;
    for (int k = 0; k < degree; ++k) {
        float a = v * f;
        o[dims * (1 + 2 * k) + j] = sinf(a);
        o[dims * (2 + 2 * k) + j] = cosf(a);
        f *= 2.f;
    }
}

}  // namespace
}  // namespace srf

using namespace srf;

extern "C" int srf_ndc_rays(const float* rays_o, const float* rays_d, const float* fx, const float* fy, int n_rays,
                            int height, int width, float near_plane, float* rays_o_ndc, float* rays_d_ndc,
                            float* vdirs, void* stream) {
    if (!rays_d || n_rays < 0) return rays_d ? SRF_ERR_SHAPE : SRF_ERR_NULL;
    if ((rays_o_ndc || rays_d_ndc) && (!rays_o || !fx || !fy)) return SRF_ERR_NULL;
    if (n_rays == 0) return SRF_OK;
    ndc_rays_kernel<<<grid_1d(n_rays, 256), 256, 0, as_stream(stream)>>>(
        rays_o, rays_d, fx, fy, n_rays, float(height), float(width), near_plane, rays_o_ndc, rays_d_ndc, vdirs);
    return launch_status();
}

extern "C" int srf_pixel_rays(const int32_t* pixel_id, const float* intrinsics, const float* extrinsics, int n_rays,
                              int half_pixel, float* rays_o, float* rays_d, void* stream) {
    if (!pixel_id || !intrinsics || !extrinsics || !rays_o || !rays_d) return SRF_ERR_NULL;
    if (n_rays < 0) return SRF_ERR_SHAPE;
    if (n_rays == 0) return SRF_OK;
    pixel_rays_kernel<<<grid_1d(n_rays, 256), 256, 0, as_stream(stream)>>>(pixel_id, intrinsics, extrinsics, n_rays,
                                                                          half_pixel, rays_o, rays_d);
    return launch_status();
}

extern "C" int srf_stratified_z(float* z, const float* u, int n_rays, int n_samples, float near_plane,
                                float far_plane, int lindisp, void* stream) {
    if (!z) return SRF_ERR_NULL;
    if (n_rays < 0 || n_samples < 1) return SRF_ERR_SHAPE;
    if (n_rays == 0) return SRF_OK;
    int64_t tot = int64_t(n_rays) * n_samples;
    stratified_kernel<<<grid_1d(tot, 256), 256, 0, as_stream(stream)>>>(z, u, n_rays, n_samples, near_plane,
                                                                        far_plane, lindisp);
    return launch_status();
}

extern "C" int srf_sample_pdf(float* samples, const float* bins, const float* weights, const float* u, int n_rays,
                              int n_bins, int n_samples, void* stream) {
    if (!samples || !bins || !weights) return SRF_ERR_NULL;
    // 4 warps x (cdf + bins) x n_bins floats must fit the default 48 KB of shared memory
    if (n_rays < 0 || n_bins < 2 || n_bins > 1536 || n_samples < 1) return SRF_ERR_SHAPE;
    if (n_rays == 0) return SRF_OK;
    const int warps = 4;
    size_t smem = size_t(warps) * 2 * n_bins * sizeof(float);
    sample_pdf_kernel<<<grid_1d(n_rays, warps), warps * 32, smem, as_stream(stream)>>>(samples, bins, weights, u,
                                                                                      n_rays, n_bins, n_samples);
    return launch_status();
}

extern "C" int srf_fine_z(float* z_fine, const float* z_coarse, const float* weights_coarse, const float* u,
                          int n_rays, int n_coarse, int n_fine, void* stream) {
    if (!z_fine || !z_coarse || !weights_coarse) return SRF_ERR_NULL;
    if (n_rays < 0 || n_coarse < 3 || n_fine < 1 || n_coarse + n_fine > 1024) return SRF_ERR_SHAPE;
    if (n_rays == 0) return SRF_OK;
    const int warps = 4;
    size_t smem = size_t(warps) * (2 * (n_coarse - 1) + n_coarse + n_fine) * sizeof(float);
    fine_z_kernel<<<grid_1d(n_rays, warps), warps * 32, smem, as_stream(stream)>>>(z_fine, z_coarse, weights_coarse,
                                                                                  u, n_rays, n_coarse, n_fine);
    return launch_status();
}

extern "C" int srf_aabb_z(float* z, const float* rays_o, const float* rays_d, const float* u, int n_rays,
                          int n_samples, const float* bbox, float near_plane, float far_plane, float step_size,
                          void* stream) {
    if (!z || !rays_o || !rays_d || !bbox) return SRF_ERR_NULL;
    if (n_rays < 0 || n_samples < 1) return SRF_ERR_SHAPE;
    if (n_rays == 0) return SRF_OK;
    int64_t tot = int64_t(n_rays) * n_samples;
    aabb_z_kernel<<<grid_1d(tot, 256), 256, 0, as_stream(stream)>>>(z, rays_o, rays_d, u, n_rays, n_samples, bbox[0],
                                                                    bbox[1], bbox[2], bbox[3], bbox[4], bbox[5],
                                                                    near_plane, far_plane, step_size);
    return launch_status();
}

extern "C" int srf_positional_encoding(float* out, int ld_out, const float* x, int64_t m, int dims, int degree,
                                       void* stream) {
    if (!out || !x) return SRF_ERR_NULL;
    if (m < 0 || dims < 1 || degree < 0 || degree > 24 || ld_out < dims * (2 * degree + 1)) return SRF_ERR_SHAPE;
    if (m == 0) return SRF_OK;
    pe_kernel<<<grid_1d(m * dims, 256), 256, 0, as_stream(stream)>>>(out, ld_out, x, m, dims, degree);
    return launch_status();
}
