// TensoRF grid maintenance: the alpha mask's 3^3 max-pool and threshold with the
// occupied box (SimpleTensoRF09.py:859-876), bilinear resampling of planes and
// lines to a new resolution (upsample_vectors_and_matrices, :1284-1301) and the
// crop of planes and lines to a sub-box (shrink_tensor, :1303-1320).  Planes and
// lines are channels-last (plane (H, W, R), line (L, 1, R)), as the VM lookups
// store them.
#include <climits>

#include "srf_common.cuh"

namespace srf {
namespace {

// max_pool3d(kernel 3, padding 1, stride 1) of alpha[z][y][x], then alpha >=
// threshold -> 1 else 0.  bounds[0..2] collect max(g - 1 - i) and bounds[3..5]
// max(i) over the occupied nodes per axis (x, y, z), so that a memset to -1
// initialises all six; a warp reduces before its one atomic per bound.
__global__ void pool_threshold_kernel(const float* __restrict__ a, int gx, int gy, int gz, float thr,
                                      float* __restrict__ out, int* __restrict__ bounds) {
    int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t n = int64_t(gx) * gy * gz;
    bool occ = false;
    int x = 0, y = 0, z = 0;
    if (t < n) {
        x = int(t % gx);
        y = int((t / gx) % gy);
        z = int(t / (int64_t(gx) * gy));
        float m = -INFINITY;
        for (int dz = -1; dz <= 1; ++dz) {
            int zz = z + dz;
            if (zz < 0 || zz >= gz) continue;
            for (int dy = -1; dy <= 1; ++dy) {
                int yy = y + dy;
                if (yy < 0 || yy >= gy) continue;
                const float* row = a + (int64_t(zz) * gy + yy) * gx;
                for (int dx = -1; dx <= 1; ++dx) {
                    int xx = x + dx;
                    if (xx < 0 || xx >= gx) continue;
                    m = fmaxf(m, row[xx]);
                }
            }
        }
        occ = m >= thr;
        out[t] = occ ? 1.f : 0.f;
    }
    const unsigned act = __ballot_sync(0xffffffffu, occ);
    if (!act) return;
    const int v[6] = {gx - 1 - x, gy - 1 - y, gz - 1 - z, x, y, z};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        int r = __reduce_max_sync(0xffffffffu, occ ? v[k] : -1);
        if ((threadIdx.x & 31) == 0) atomicMax(bounds + k, r);
    }
}

// torch's bilinear upsampling with align_corners=True (CPU kernel of
// F.interpolate): source index scale * i with scale = (in - 1) / (out - 1),
// lower index clamped to in - 1, weight of the upper one clamped to [0, 1], the
// same index when the size is unchanged; rows weighted after columns.
struct Lerp {
    int i0, i1;
    float w0, w1;
};

__device__ __forceinline__ Lerp lerp_index(int o, int in, int out) {
    Lerp l;
    if (in == out) {
        l.i0 = l.i1 = o;
        l.w0 = 1.f;
        l.w1 = 0.f;
        return l;
    }
    const float scale = out > 1 ? float(in - 1) / float(out - 1) : 0.f;
    const float real = __fmul_rn(scale, float(o));
    int i0 = int(floorf(real));
    i0 = i0 < in - 1 ? i0 : in - 1;
    float w1 = fminf(fmaxf(__fsub_rn(real, float(i0)), 0.f), 1.f);
    l.i0 = i0;
    l.i1 = i0 + (i0 < in - 1 ? 1 : 0);
    l.w1 = w1;
    l.w0 = __fsub_rn(1.f, w1);
    return l;
}

__global__ void resample_kernel(const float* __restrict__ src, int h, int w, int r, float* __restrict__ dst, int h2,
                                int w2) {
    int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= int64_t(h2) * w2 * r) return;
    const int c = int(t % r);
    const int x = int((t / r) % w2);
    const int y = int(t / (int64_t(r) * w2));
    const Lerp ly = lerp_index(y, h, h2), lx = lerp_index(x, w, w2);
    auto at = [&](int yy, int xx) { return src[(int64_t(yy) * w + xx) * r + c]; };
    float t0 = __fadd_rn(__fmul_rn(at(ly.i0, lx.i0), lx.w0), __fmul_rn(at(ly.i0, lx.i1), lx.w1));
    float t1 = __fadd_rn(__fmul_rn(at(ly.i1, lx.i0), lx.w0), __fmul_rn(at(ly.i1, lx.i1), lx.w1));
    dst[t] = __fadd_rn(__fmul_rn(t0, ly.w0), __fmul_rn(t1, ly.w1));
}

__global__ void crop_kernel(const float* __restrict__ src, int w, int r, int row0, int col0, float* __restrict__ dst,
                            int h2, int w2) {
    int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= int64_t(h2) * w2 * r) return;
    const int c = int(t % r);
    const int x = int((t / r) % w2);
    const int y = int(t / (int64_t(r) * w2));
    dst[t] = src[(int64_t(y + row0) * w + (x + col0)) * r + c];
}

}  // namespace
}  // namespace srf

using namespace srf;

extern "C" int srf_alpha_pool_threshold(const float* alpha, int gx, int gy, int gz, float threshold, float* volume,
                                        int32_t* bounds, void* stream) {
    if (!alpha || !volume || !bounds) return SRF_ERR_NULL;
    if (gx < 1 || gy < 1 || gz < 1) return SRF_ERR_SHAPE;
    cudaStream_t s = as_stream(stream);
    cudaError_t e = cudaMemsetAsync(bounds, 0xff, 6 * sizeof(int32_t), s);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return SRF_ERR_CUDA;
    }
    int64_t n = int64_t(gx) * gy * gz;
    pool_threshold_kernel<<<grid_1d(n, 256), 256, 0, s>>>(alpha, gx, gy, gz, threshold, volume, bounds);
    return launch_status();
}

extern "C" int srf_resample_grid(const float* src, int h, int w, int comps, float* dst, int h_new, int w_new,
                                 void* stream) {
    if (!src || !dst) return SRF_ERR_NULL;
    if (h < 1 || w < 1 || comps < 1 || h_new < 1 || w_new < 1) return SRF_ERR_SHAPE;
    int64_t n = int64_t(h_new) * w_new * comps;
    resample_kernel<<<grid_1d(n, 256), 256, 0, as_stream(stream)>>>(src, h, w, comps, dst, h_new, w_new);
    return launch_status();
}

extern "C" int srf_crop_grid(const float* src, int h, int w, int comps, int row0, int col0, float* dst, int h_new,
                             int w_new, void* stream) {
    if (!src || !dst) return SRF_ERR_NULL;
    if (h < 1 || w < 1 || comps < 1 || h_new < 1 || w_new < 1 || row0 < 0 || col0 < 0 || row0 + h_new > h ||
        col0 + w_new > w)
        return SRF_ERR_SHAPE;
    int64_t n = int64_t(h_new) * w_new * comps;
    crop_kernel<<<grid_1d(n, 256), 256, 0, as_stream(stream)>>>(src, w, comps, row0, col0, dst, h_new, w_new);
    return launch_status();
}
