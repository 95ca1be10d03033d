// Training-batch assembly on the device (DataPreprocessor10.select_batch_indices /
// load_nerf_cached_batch, src/data_preprocessors/DataPreprocessor10.py:496-549):
// every epoch visits the cached rays in a fresh random order, in consecutive
// slices of n_rays, and the selected rays' pixel ids, colours and cameras are
// gathered into the step's input buffers.  The order is a keyed bijection of
// [0, pool) (a four-round Feistel network on the next power-of-four domain with
// cycle walking), so no permutation is stored or shuffled: batch b of the run
// takes positions ((b mod B) n, ...) of epoch b div B's order, B = pool div n
// full batches per epoch.  The batch counter lives on the device, so a captured
// training step replays with a new batch every time.
#include "srf_common.cuh"

namespace srf {
namespace {

// 32-bit integer mixer ("lowbias32", C. Wellons' hash-prospector search).
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

struct Perm {
    uint32_t keys[4];
    int half;          // bits per Feistel half
    uint32_t mask;     // (1 << half) - 1
    int64_t size;      // the permuted range [0, size)
};

__device__ __forceinline__ Perm make_perm(int64_t size, uint64_t seed, int64_t epoch) {
    Perm p;
    int bits = 2;
    while ((int64_t(1) << bits) < size) ++bits;
    p.half = (bits + 1) / 2;
    p.mask = (1u << p.half) - 1u;
    p.size = size;
    const uint32_t s0 = uint32_t(seed), s1 = uint32_t(seed >> 32);
    for (int r = 0; r < 4; ++r)
        p.keys[r] = mix32(s0 ^ mix32(uint32_t(epoch) * 4u + uint32_t(r) + mix32(s1 ^ uint32_t(epoch >> 32))));
    return p;
}

__device__ __forceinline__ uint32_t feistel(uint32_t x, const Perm& p) {
    uint32_t l = x >> p.half, r = x & p.mask;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t t = l ^ (mix32(r ^ p.keys[k]) & p.mask);
        l = r;
        r = t;
    }
    return (l << p.half) | r;
}

// Position -> element of [0, size): walk the Feistel cycle until it lands inside
// the range (the domain is < 4 size, so about 2 steps on average).  The walk is
// capped; a capped walk (not expected in practice) raises the device flag.
constexpr int kMaxWalk = 4096;

__device__ __forceinline__ int64_t permute(int64_t pos, const Perm& p, int* flag) {
    uint32_t y = uint32_t(pos);
    for (int i = 0; i < kMaxWalk; ++i) {
        y = feistel(y, p);
        if (int64_t(y) < p.size) return y;
    }
    raise_flag(flag, kFlagRange);
    return pos;
}

__global__ void batch_assemble_kernel(const int32_t* __restrict__ pool_rows, const int32_t* __restrict__ pool_pid,
                                      const float* __restrict__ pool_val, int channels, int64_t pool,
                                      int64_t table_rows, int n, uint64_t seed,
                                      const int32_t* __restrict__ counter, const float* __restrict__ intr,
                                      const float* __restrict__ extr, int n_views, int32_t* __restrict__ out_pid,
                                      float* __restrict__ out_val, int32_t* __restrict__ out_idx,
                                      float* __restrict__ out_intr, float* __restrict__ out_extr, int* flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t per_epoch = pool / n;
    const int64_t b = counter ? int64_t(*counter) : 0;
    const int64_t epoch = b / per_epoch;
    const int64_t pos = (b % per_epoch) * n + i;
    const Perm p = make_perm(pool, seed, epoch);
    int64_t j = pool_rows ? int64_t(pool_rows[permute(pos, p, flag)]) : permute(pos, p, flag);
    if (j < 0 || j >= table_rows) {   // a bad entry of pool_rows: gather row 0 and raise the flag
        raise_flag(flag, kFlagRange);
        j = 0;
    }
    if (out_idx) out_idx[i] = int32_t(j);
    int32_t img = 0;
    if (pool_pid) {
        img = pool_pid[3 * j];
        out_pid[3 * i] = img;
        out_pid[3 * i + 1] = pool_pid[3 * j + 1];
        out_pid[3 * i + 2] = pool_pid[3 * j + 2];
    }
    for (int c = 0; c < channels; ++c) out_val[int64_t(i) * channels + c] = pool_val[j * channels + c];
    if (intr || extr) {
        if (img < 0 || img >= n_views) {
            raise_flag(flag, kFlagRange);
            img = 0;
        }
        if (intr)
            for (int k = 0; k < 9; ++k) out_intr[9 * i + k] = intr[9 * img + k];
        if (extr)
            for (int k = 0; k < 16; ++k) out_extr[16 * i + k] = extr[16 * img + k];
    }
}

// Counter-based uniforms in [0, 1): u[i] = top 24 bits of a hash of (seed, draw, i),
// draw = *counter (the step count) when given.  Each (seed, draw) gives a fresh
// stream, so a captured step draws new uniforms on every replay.
__global__ void uniforms_kernel(float* __restrict__ u, int64_t n, uint64_t seed, const int32_t* __restrict__ counter,
                                int stream_id) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t draw = counter ? uint32_t(*counter) : 0u;
    uint32_t h = mix32(uint32_t(seed) ^ mix32(draw * 0x9e3779b9u + uint32_t(stream_id)));
    h = mix32(h ^ mix32(uint32_t(seed >> 32) + uint32_t(i)));
    h = mix32(h ^ uint32_t(i >> 32));
    u[i] = float(h >> 8) * (1.f / 16777216.f);
}

}  // namespace
}  // namespace srf

using namespace srf;

extern "C" int srf_batch_assemble(const int32_t* pool_rows, const int32_t* pool_pixel_id, const float* pool_values,
                                  int channels, int64_t pool_size, int64_t table_rows, int n_rays, uint64_t seed,
                                  const int32_t* batch_counter_dev,
                                  const float* intrinsics, const float* extrinsics, int n_views,
                                  int32_t* out_pixel_id, float* out_values, int32_t* out_index,
                                  float* out_intrinsics, float* out_extrinsics, void* stream) {
    if (n_rays < 1 || pool_size < n_rays || pool_size > (int64_t(1) << 30) || channels < 0 || channels > 16 ||
        table_rows < 1 || (!pool_rows && table_rows < pool_size))
        return SRF_ERR_SHAPE;
    if (pool_pixel_id && !out_pixel_id) return SRF_ERR_NULL;
    if (channels > 0 && (!pool_values || !out_values)) return SRF_ERR_NULL;
    if ((intrinsics && !out_intrinsics) || (extrinsics && !out_extrinsics)) return SRF_ERR_NULL;
    if ((intrinsics || extrinsics) && (!pool_pixel_id || n_views < 1)) return SRF_ERR_SHAPE;
    batch_assemble_kernel<<<grid_1d(n_rays, 256), 256, 0, as_stream(stream)>>>(
        pool_rows, pool_pixel_id, pool_values, channels, pool_size, table_rows, n_rays, seed, batch_counter_dev, intrinsics, extrinsics,
        n_views, out_pixel_id, out_values, out_index, out_intrinsics, out_extrinsics, device_flag());
    return launch_status();
}

extern "C" int srf_uniforms(float* u, int64_t n, uint64_t seed, const int32_t* counter_dev, int stream_id,
                            void* stream) {
    if (!u) return SRF_ERR_NULL;
    if (n < 0) return SRF_ERR_SHAPE;
    if (n == 0) return SRF_OK;
    uniforms_kernel<<<grid_1d(n, 256), 256, 0, as_stream(stream)>>>(u, n, seed, counter_dev, stream_id);
    return launch_status();
}
