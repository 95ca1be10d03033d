// Fused forward of a whole NeRF MLP (SimpleNeRF17.py:696-785) on tcgen05: every
// trunk layer (with the skip concat), the sigma head, the feature layer, the
// view layer and the rgb head in one persistent kernel, after the positional
// encodings (written by the standalone encoder: 256 bytes a sample, which the
// backward reads anyway).  A CTA takes 128 samples at a time and keeps their
// activations in shared memory from the encodings to the heads; only the layer
// weights move, streamed from L2 by TMA, one 64-column K block per stage.
//
//   shared memory: ACT  4 x [128 rows x 64 columns] 16-bit, 128-byte swizzle:
//                       the current layer's input, overwritten by its output
//                  ENC  [128 x 64]: PE(points) of the tile (TMA; the next tile's is
//                       loaded once the skip layer, its last reader, is done)
//                  VX   [128 x 64]: PE(view dirs) of the tile (TMA)
//                  W    kFusedStages x [<= 256 rows x 64 columns]: weight K blocks
//   tensor memory: two FP32 accumulators of 256 columns; layer g of the CTA's
//                  sequence accumulates in g % 2.
//
// Warp roles (320 threads): warp 0 loads weight K blocks and encodings (TMA), warp 1 issues
// the MMAs, warps 2..9 drain the accumulators.  Warp w reads tensor-memory lane
// quadrant w % 4 (32 rows) and, of each 64-column block, the 32 columns of half
// (w - 2) / 4, blocks in order: block b of a layer's output is complete after
// b + 1 of the epilogue's 4 steps and releases the next layer's MMAs on that K
// block (act_ready), so the next layer runs while the epilogue still drains the
// previous one.  An epilogue step adds the bias, applies the ReLU, rounds to
// the operand format and writes over ACT.  Each layer kind (plain, with a head,
// without ReLU, the 128-wide view layer) is its own compiled instance.
//
// Forward-only calls store nothing but the heads (raw sigma, sigma, rgb).  With
// STORE, every activation the backward reads (each layer's output, the ReLU bit
// masks) also goes to global memory straight from the epilogue registers, so
// each activation crosses HBM once (written) instead of twice (written, then
// read by the next layer).
//
// Every mbarrier wait is bounded; a timeout sets the abort flag, the roles stop
// issuing work, drain what they started, free tensor memory and report through
// the device error flag.
#pragma once

#include "tc_gemm.cuh"

namespace srf {
namespace tc {

constexpr int kFusedMaxLayers = 10;
constexpr int kFusedStages = 3;
constexpr int kFusedThreads = 320;
constexpr uint32_t kActBlockBytes = 128 * 128;   // 128 rows x 64 16-bit columns
constexpr uint32_t kWStageBytes = 256 * 128;     // up to 256 weight rows x 64 16-bit columns
constexpr int kFusedBiasFloats = 9 * 256 + 128;   // the biases of 8 trunk layers, the feature and the view layer
constexpr int kFusedHeadFloats = 1024;
constexpr size_t kFusedSmem = 1024 + 6 * size_t(kActBlockBytes) + size_t(kFusedStages) * kWStageBytes +
                              (size_t(kFusedBiasFloats) + kFusedHeadFloats + 4 * kFusedMaxLayers) * 4 +
                              2 * 128 * 4 * 4 + 256;
static_assert(31 * 8 <= 256, "barriers of the fused MLP kernel");
static_assert(kFusedSmem <= 232448, "shared memory of the fused MLP kernel");

// Layer kinds, one compiled epilogue each.
enum : int {
    kFusedPlain = 0,       // 256 outputs, ReLU
    kFusedSigma = 1,       // 256 outputs, ReLU, sigma head
    kFusedLinear = 2,      // 256 outputs, no ReLU (the feature layer)
    kFusedView = 3,        // 128 outputs, ReLU, rgb head (the view layer, always last)
    kFusedSigmaRgb = 4,    // 256 outputs, ReLU, sigma + rgb heads (no view branch, always last)
};

struct FusedLayer {
    int kind;
    int kb;          // 64-wide K blocks of the input
    int ext_kb;      // which of them is an encoding slab (-1: none); the others are ACT blocks 0.. in order
    int ext_src;     // that slab: 0 ENC, 1 VX
    int ext_wait;    // the slab holds a new encoding for this layer (the MMA waits for it)
    int n;           // outputs: 256, or 128 for the view layer
    int head;        // kHeadNone / kHeadSigma / kHeadRgb / kHeadSigmaRgb
    int enc_last;    // the last layer that reads ENC: its MMAs release ENC for the next tile
    int bias_off;    // offset of the bias in the shared bias array
    int head_off;    // offset of the head weights (units x n) in the shared head array
};

struct FusedProgram {
    int nl;
    int fmt;
    int has_vx;            // the view layer reads VX
    int has_noise;
    int64_t M;
    FusedLayer layer[kFusedMaxLayers];
    const float* bias[kFusedMaxLayers];
    const float* head_w[kFusedMaxLayers];
    const float* head_b[kFusedMaxLayers];
    uint32_t* bits_out[kFusedMaxLayers];   // STORE: [M, n / 32] or NULL
    uint16_t* out[kFusedMaxLayers];        // STORE: [M, n] or NULL
    int enc_at, vx_at;     // the producer loads ENC of the next tile before the weights of layer enc_at
                           // (nl: after the tile's last layer), VX of the tile before those of layer vx_at
    const float* noise;    // [M] added to the raw sigma
    float* sraw;           // [M]
    float* sigma;          // [M]
    float* rgb_ws;         // [M, 3]
    float* rgb_out;        // [M, 3]
    int* found_inf;
    int* flag;
};

// Tensor maps of the 16-bit packed weights of each layer (n x K, boxes of 64 x n)
// and of the two encodings ([M, 64], boxes of 64 x 128).
struct FusedMaps {
    CUtensorMap w[kFusedMaxLayers];
    CUtensorMap enc, vx;
};

// max that keeps a NaN operand (an overflow check must see NaNs)
__device__ __forceinline__ float max_nan(float a, float b) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}

// Per-thread state of the epilogue warps.
struct FusedEpi {
    int q, half, lane, r;     // lane quadrant, column half, lane, row of the tile
    int64_t m;                // sample
    bool live;
    float mx;                 // largest stored magnitude (NaN when one was NaN)
};

// Step i of one layer's epilogue for this warp: columns 64 i + 32 half .. + 31 of
// its 32 rows from the accumulator registers rr: bias, ReLU, head partial dot
// products, the 16-bit result into ACT block i and, with STORE, to global memory
// with the ReLU bits; then block i is released to the next layer.
template <bool STORE, int N, bool RELU, int UNITS>
__device__ __forceinline__ void fused_step(const FusedProgram& P, int l, bool act_out, int i, const uint32_t (&rr)[32],
                                           uint8_t* act, const float* bias, const float* hw, uint64_t* act_ready,
                                           FusedEpi& e, float (&hp)[4], bool check) {
    const int c = 2 * i + e.half;   // 32-column chunk
    const int f = P.fmt;
    float v[32];
    const float4* b4 = reinterpret_cast<const float4*>(bias + c * 32);
#pragma unroll
    for (int g = 0; g < 8; ++g) {
        const float4 b = b4[g];
        v[4 * g] = __uint_as_float(rr[4 * g]) + b.x;
        v[4 * g + 1] = __uint_as_float(rr[4 * g + 1]) + b.y;
        v[4 * g + 2] = __uint_as_float(rr[4 * g + 2]) + b.z;
        v[4 * g + 3] = __uint_as_float(rr[4 * g + 3]) + b.w;
    }
    if (RELU) {
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = fmaxf(v[j], 0.f);
    }
    if (STORE && P.bits_out[l] && e.live) {
        uint32_t mb = 0u;
#pragma unroll
        for (int j = 0; j < 32; ++j) mb |= uint32_t(v[j] > 0.f) << j;
        P.bits_out[l][e.m * (N / 32) + c] = mb;
    }
#pragma unroll
    for (int u = 0; u < UNITS; ++u) {
        // four independent partial sums (short dependency chains), then their sum
        const float4* w4 = reinterpret_cast<const float4*>(hw + u * N + c * 32);
        float s4[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int g = 0; g < 8; ++g) {
            const float4 w = w4[g];
            s4[0] += v[4 * g] * w.x;
            s4[1] += v[4 * g + 1] * w.y;
            s4[2] += v[4 * g + 2] * w.z;
            s4[3] += v[4 * g + 3] * w.w;
        }
        hp[u] += (s4[0] + s4[1]) + (s4[2] + s4[3]);
    }
    if (check) {
        float m4[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int j = 0; j < 32; ++j) m4[j & 3] = max_nan(m4[j & 3], fabsf(v[j]));
        e.mx = max_nan(e.mx, max_nan(max_nan(m4[0], m4[1]), max_nan(m4[2], m4[3])));
    }
    if (act_out || (STORE && e.live)) {
        uint8_t* row = act + size_t(i) * kActBlockBytes + e.r * 128;
        uint4* dst = STORE && e.live ? reinterpret_cast<uint4*>(P.out[l] + e.m * N + c * 32) : nullptr;
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            const uint4 pk = make_uint4(pack16(v[8 * g], v[8 * g + 1], f), pack16(v[8 * g + 2], v[8 * g + 3], f),
                                        pack16(v[8 * g + 4], v[8 * g + 5], f), pack16(v[8 * g + 6], v[8 * g + 7], f));
            if (act_out) *reinterpret_cast<uint4*>(row + ((((e.half * 4 + g) ^ (e.r & 7))) << 4)) = pk;
            if (dst) dst[g] = pk;
        }
    }
    if (act_out) {
        fence_proxy_async_smem();
        __syncwarp();
        if (e.lane == 0) mbar_arrive(&act_ready[i]);
    }
}

// One layer's epilogue for this warp, steps in block order with the next step's
// tensor-memory load in flight under the current step's math.
template <bool STORE, int N, bool RELU, int UNITS>
__device__ __forceinline__ void fused_epilogue(const FusedProgram& P, int l, bool act_out, uint32_t tbase,
                                               uint8_t* act, const float* bias, const float* hw, uint64_t* act_ready,
                                               FusedEpi& e, float (&hp)[4]) {
    constexpr int HS = N / 64;   // steps
    const bool check = P.found_inf && e.live && (act_out || STORE);
    uint32_t ra[32], rb[32];
    tmem_ld_32x32b_x32(tbase + uint32_t(e.half * 32), ra);
    tmem_ld_wait();
#pragma unroll 1
    for (int i = 0; i < HS; i += 2) {
        tmem_ld_32x32b_x32(tbase + uint32_t((2 * (i + 1) + e.half) * 32), rb);
        fused_step<STORE, N, RELU, UNITS>(P, l, act_out, i, ra, act, bias, hw, act_ready, e, hp, check);
        tmem_ld_wait();
        if (i + 2 < HS) tmem_ld_32x32b_x32(tbase + uint32_t((2 * (i + 2) + e.half) * 32), ra);
        fused_step<STORE, N, RELU, UNITS>(P, l, act_out, i + 1, rb, act, bias, hw, act_ready, e, hp, check);
        tmem_ld_wait();
    }
}

template <bool STORE>
__global__ void __launch_bounds__(kFusedThreads, 1)
    mlp_fused_kernel(const __grid_constant__ FusedMaps maps, const FusedProgram P) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* act = base;
    uint8_t* enc = act + 4 * kActBlockBytes;
    uint8_t* vx = enc + kActBlockBytes;
    uint8_t* wst = vx + kActBlockBytes;
    float* sbias = reinterpret_cast<float*>(wst + size_t(kFusedStages) * kWStageBytes);
    float* shw = sbias + kFusedBiasFloats;
    float* shb = shw + kFusedHeadFloats;        // [layer][4]
    float* shx = shb + 4 * kFusedMaxLayers;     // [2 slots][128 rows][4]: half 1's head partial sums
    uint64_t* bars = reinterpret_cast<uint64_t*>(shx + 2 * 128 * 4);
    uint64_t* wfull = bars;             // [kFusedStages]
    uint64_t* wempty = bars + 4;        // [kFusedStages]
    uint64_t* acc_full = bars + 8;      // [2]
    uint64_t* acc_empty = bars + 10;    // [2]
    uint64_t* act_ready = bars + 12;    // [4]
    uint64_t* enc_full = bars + 16;
    uint64_t* vx_full = bars + 17;
    uint64_t* done = bars + 18;
    uint64_t* hx_ready = bars + 19;     // [2 slots][4 quadrants]
    uint64_t* enc_empty = bars + 27;
    uint64_t* vx_empty = bars + 28;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 29);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 30);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t num_tiles = (P.M + 127) / 128;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kFusedStages; ++s) {
            mbar_init(&wfull[s], 1);
            mbar_init(&wempty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(&acc_full[a], 1);
            mbar_init(&acc_empty[a], 256);
        }
        for (int b = 0; b < 4; ++b) mbar_init(&act_ready[b], 8);
        mbar_init(enc_full, 1);
        mbar_init(vx_full, 1);
        mbar_init(enc_empty, 1);
        mbar_init(vx_empty, 1);
        mbar_init(done, 1);
        for (int i = 0; i < 8; ++i) mbar_init(&hx_ready[i], 32);
        *abort_flag = 0;
        fence_barrier_init();
    }
    for (int l = 0; l < P.nl; ++l) {
        const FusedLayer& L = P.layer[l];
        for (int i = threadIdx.x; i < L.n; i += blockDim.x) sbias[L.bias_off + i] = P.bias[l][i];
        const int units = head_units(L.head);
        for (int i = threadIdx.x; i < units * L.n; i += blockDim.x) shw[L.head_off + i] = P.head_w[l][i];
        if (threadIdx.x < 4) shb[4 * l + threadIdx.x] = int(threadIdx.x) < units ? P.head_b[l][threadIdx.x] : 0.f;
    }
    if (warp == 1) {
        tmem_alloc(tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---------------------------------------- weight and encoding producer
        for (int l = 0; l < P.nl; ++l) prefetch_tmap(&maps.w[l]);
        prefetch_tmap(&maps.enc);
        if (P.has_vx) prefetch_tmap(&maps.vx);
        uint32_t it = 0, t = 0, enc_loads = 0, vx_loads = 0;
        uint32_t last_parity[kFusedStages] = {};
        bool used[kFusedStages] = {};
        bool ok = true;
        // ENC / VX of tile `tile` (the n-th load of that slab) once the MMAs that read the
        // previous contents are done; every copy is waited for before the CTA exits
        auto load_enc = [&](int64_t tile, uint32_t n) {
            if (n > 0 && !mbar_wait_sleep(enc_empty, (n - 1) & 1, abort_flag)) return false;
            mbar_arrive_expect_tx(enc_full, kActBlockBytes);
            tma_load_2d(enc, &maps.enc, enc_full, 0, int32_t(tile * 128));
            ++enc_loads;
            return true;
        };
        auto load_vx = [&](int64_t tile, uint32_t n) {
            if (n > 0 && !mbar_wait_sleep(vx_empty, (n - 1) & 1, abort_flag)) return false;
            mbar_arrive_expect_tx(vx_full, kActBlockBytes);
            tma_load_2d(vx, &maps.vx, vx_full, 0, int32_t(tile * 128));
            ++vx_loads;
            return true;
        };
        if (int64_t(blockIdx.x) < num_tiles) ok = load_enc(blockIdx.x, 0);
        for (int64_t tile = blockIdx.x; ok && tile < num_tiles; tile += gridDim.x, ++t) {
            const int64_t next = tile + gridDim.x;
            for (int l = 0; ok && l <= P.nl; ++l) {
                if (l == P.enc_at && next < num_tiles && !load_enc(next, t + 1)) ok = false;
                if (ok && P.has_vx && l == P.vx_at && !load_vx(tile, t)) ok = false;
                if (!ok || l == P.nl) break;
                const FusedLayer& L = P.layer[l];
                for (int kb = 0; kb < L.kb; ++kb, ++it) {
                    const int s = int(it % kFusedStages);
                    const uint32_t ph = (it / kFusedStages) & 1;
                    if (!mbar_wait_sleep(&wempty[s], ph ^ 1, abort_flag)) {
                        ok = false;
                        break;
                    }
                    mbar_arrive_expect_tx(&wfull[s], uint32_t(L.n) * 128);
                    tma_load_2d(wst + size_t(s) * kWStageBytes, &maps.w[l], &wfull[s], kb * 64, 0);
                    used[s] = true;
                    last_parity[s] = ph;
                }
            }
        }
        if (!ok) *abort_flag = 1;
        // every copy this thread started has landed before the CTA may exit
        for (int s = 0; s < kFusedStages; ++s)
            if (used[s] && !mbar_wait_sleep(&wfull[s], last_parity[s], nullptr)) *abort_flag = 1;
        if (enc_loads && !mbar_wait_sleep(enc_full, (enc_loads - 1) & 1, nullptr)) *abort_flag = 1;
        if (vx_loads && !mbar_wait_sleep(vx_full, (vx_loads - 1) & 1, nullptr)) *abort_flag = 1;
    } else if (warp == 1 && lane == 0) {
        // ------------------------------------------------------------------ MMA
        uint32_t it = 0, g = 0, act_seq = 0, enc_seq = 0, vx_seq = 0;   // enc / vx: loads consumed
        bool ok = true;
        for (int64_t tile = blockIdx.x; ok && tile < num_tiles; tile += gridDim.x) {
            for (int l = 0; ok && l < P.nl; ++l, ++g) {
                const FusedLayer& L = P.layer[l];
                const uint32_t a = g & 1;
                if (!mbar_wait_sleep(&acc_empty[a], ((g >> 1) & 1) ^ 1, abort_flag)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t idesc = idesc_f16(128, L.n, 0, 0, P.fmt);
                const uint32_t d_tmem = tmem + a * 256;
                int ab = 0;
                for (int kb = 0; kb < L.kb; ++kb, ++it) {
                    uint32_t a_addr;
                    if (kb == L.ext_kb) {
                        if (L.ext_wait) {
                            uint64_t* rdy = L.ext_src ? vx_full : enc_full;
                            uint32_t& seq = L.ext_src ? vx_seq : enc_seq;
                            if (!mbar_wait_sleep(rdy, seq & 1, abort_flag)) {
                                ok = false;
                                break;
                            }
                            ++seq;
                        }
                        a_addr = smem_u32(L.ext_src ? vx : enc);
                    } else {
                        if (!mbar_wait_sleep(&act_ready[ab], act_seq & 1, abort_flag)) {
                            ok = false;
                            break;
                        }
                        a_addr = smem_u32(act + size_t(ab) * kActBlockBytes);
                        ++ab;
                    }
                    const int s = int(it % kFusedStages);
                    if (!mbar_wait_sleep(&wfull[s], (it / kFusedStages) & 1, abort_flag)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t b_addr = smem_u32(wst + size_t(s) * kWStageBytes);
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const uint64_t ad = smem_desc(a_addr + k * 32, 0, 1024, kSwizzle128B);
                        const uint64_t bd = smem_desc(b_addr + k * 32, 0, 1024, kSwizzle128B);
                        mma_f16(d_tmem, ad, bd, idesc, (kb | k) != 0);
                    }
                    mma_commit(&wempty[s]);
                }
                if (!ok) break;
                if (ab > 0) ++act_seq;   // the previous layer's output is consumed
                mma_commit(&acc_full[a]);
                // the slabs this layer read last are free once its MMAs complete
                if (L.enc_last) mma_commit(enc_empty);
                if (L.ext_kb >= 0 && L.ext_src) mma_commit(vx_empty);
            }
        }
        if (!ok) *abort_flag = 1;
        // all MMAs issued by this thread complete before tensor memory is freed
        mma_commit(done);
        if (!mbar_wait_sleep(done, 0, nullptr)) *abort_flag = 1;
    } else if (warp >= 2) {
        // ------------------------------------------------------------- epilogue
        FusedEpi e;
        e.q = warp & 3;
        e.half = (warp - 2) >> 2;
        e.lane = lane;
        e.r = e.q * 32 + lane;
        e.mx = 0.f;
        uint32_t g = 0, hx_seq = 0;
        bool ok = true;
        for (int64_t tile = blockIdx.x; ok && tile < num_tiles; tile += gridDim.x) {
            e.m = tile * 128 + e.r;
            e.live = e.m < P.M;
            for (int l = 0; l < P.nl; ++l, ++g) {
                const FusedLayer& L = P.layer[l];
                const uint32_t a = g & 1;
                const bool act_out = l + 1 < P.nl;
                if (!mbar_wait_sleep(&acc_full[a], (g >> 1) & 1, abort_flag)) {
                    ok = false;
                    break;
                }
                __syncwarp();
                tc_fence_after();
                const uint32_t tbase = tmem + a * 256 + (uint32_t(e.q * 32) << 16);
                const float* bias = sbias + L.bias_off;
                const float* hw = shw + L.head_off;
                float hp[4] = {0.f, 0.f, 0.f, 0.f};
                switch (L.kind) {
                    case kFusedSigma:
                        fused_epilogue<STORE, 256, true, 1>(P, l, act_out, tbase, act, bias, hw, act_ready, e, hp);
                        break;
                    case kFusedLinear:
                        fused_epilogue<STORE, 256, false, 0>(P, l, act_out, tbase, act, bias, hw, act_ready, e, hp);
                        break;
                    case kFusedView:
                        fused_epilogue<STORE, 128, true, 3>(P, l, act_out, tbase, act, bias, hw, act_ready, e, hp);
                        break;
                    case kFusedSigmaRgb:
                        fused_epilogue<STORE, 256, true, 4>(P, l, act_out, tbase, act, bias, hw, act_ready, e, hp);
                        break;
                    default:
                        fused_epilogue<STORE, 256, true, 0>(P, l, act_out, tbase, act, bias, hw, act_ready, e, hp);
                        break;
                }
                tc_fence_before();
                mbar_arrive(&acc_empty[a]);
                const int units = head_units(L.head);
                if (units) {
                    // half 1 hands its partial dot products to half 0, which adds them to its own
                    // and writes the heads.  A slot is reused two head layers later, after half 0
                    // has passed the next layer's epilogue, which needs this read done.
                    const uint32_t slot = hx_seq & 1;
                    float* x = shx + (slot * 128 + e.r) * 4;
                    uint64_t* rdy = &hx_ready[slot * 4 + e.q];
                    if (e.half == 1) {
#pragma unroll
                        for (int u = 0; u < 4; ++u) x[u] = hp[u];
                        mbar_arrive(rdy);
                    } else if (mbar_wait_sleep(rdy, (hx_seq >> 1) & 1, abort_flag)) {
#pragma unroll
                        for (int u = 0; u < 4; ++u) hp[u] += x[u];
                        if (e.live) {
                            // SimpleNeRF17.py:735-750 (sigma head + noise + ReLU) and :771-777 (sigmoid rgb)
                            const float* hb = shb + 4 * l;
                            int u0 = 0;
                            if (L.head != kHeadRgb) {
                                float sv = hp[0] + hb[0];
                                if (P.has_noise) sv += P.noise[e.m];
                                P.sraw[e.m] = sv;
                                P.sigma[e.m] = sv > 0.f ? sv : 0.f;
                                u0 = 1;
                            }
                            if (L.head != kHeadSigma) {
#pragma unroll
                                for (int cc = 0; cc < 3; ++cc) {
                                    const float rv = 1.f / (1.f + expf(-(hp[u0 + cc] + hb[u0 + cc])));
                                    P.rgb_ws[3 * e.m + cc] = rv;
                                    P.rgb_out[3 * e.m + cc] = rv;
                                }
                            }
                        }
                    } else {
                        ok = false;
                    }
                    ++hx_seq;
                    if (!ok) break;
                }
            }
        }
        if (!ok) *abort_flag = 1;
        const bool bad = !(e.mx <= fmt_max(P.fmt));
        if (P.found_inf && __any_sync(0xffffffffu, bad) && lane == 0) atomicExch(P.found_inf, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0 && *abort_flag) raise_flag(P.flag, kFlagTimeout);
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 512);
    }
}

}  // namespace tc
}  // namespace srf
