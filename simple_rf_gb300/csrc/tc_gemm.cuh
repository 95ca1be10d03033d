// Persistent tcgen05 BF16 GEMM with a fused epilogue: the tensor-core form of
// one MLP layer over a tile of 128 samples.
//
//   out[m, n] = epilogue( sum_k A[m, k] * B[n, k] ),  A = [A0 | A1] (two sources
//   along K, e.g. the skip concat [PE(x), h]), B resident in shared memory.
//
// Warp roles (192 threads): warp 0 issues TMA loads, warp 1 allocates tensor
// memory and issues tcgen05.mma (one thread), warps 2..5 drain the FP32
// accumulator from tensor memory (tcgen05.ld), apply bias / ReLU / ReLU-mask /
// rank-1 update and store BF16 rows.  Two accumulators in tensor memory let the
// epilogue of tile t overlap the MMAs of tile t+1.  Operands are K-major with the
// 128-byte swizzle that TMA writes (8-row x 128-byte atoms, SBO = 1024 B).
//
// Every mbarrier wait is bounded: on a timeout the CTA sets the device error
// flag, stops issuing work, waits (bounded) for its own copies and MMAs, frees
// its tensor memory and returns.
#pragma once

#include "tc_primitives.cuh"

namespace srf {
namespace tc {

constexpr int kBlockM = 128;
constexpr int kBlockK = 64;   // one 128-byte swizzle atom of BF16
constexpr int kThreads = 192;       // weight-gradient kernel: producer, MMA, 4 epilogue warps
// layer kernel: producer warp, MMA warp, EW epilogue warps (4: one per TMEM lane
// quadrant; 8: two per quadrant, each taking half of the columns)
constexpr int gemm_threads(int ew) { return 64 + 32 * ew; }
constexpr uint32_t kATileBytes = kBlockM * kBlockK * 2;
constexpr size_t kMaxSmem = 232448;

enum { kHeadNone = 0, kHeadSigma = 1, kHeadRgb = 2, kHeadSigmaRgb = 3 };

struct GemmEpilogue {
    const float* bias;              // [N] or NULL
    int relu;                       // apply ReLU to the result
    int fmt;                        // operand / output format (kFmtBF16, kFmtF16)
    const uint16_t* mask;           // multiply by (mask[m, n] > 0) when non-NULL
    int64_t ld_mask;
    // ReLU masks as bits, 32 columns per word: bits_out[m, c] gets bit j set where
    // stored column 32c + j is > 0 (written when non-NULL); mask_bits multiplies the
    // result by those bits (the 1-bit form of `mask`, 16x fewer bytes to read)
    uint32_t* bits_out;
    const uint32_t* mask_bits;
    int64_t ld_bits;                // words per row of both
    const float* r1_row;            // result += r1[m] * r1_col[n] (before ReLU/mask) when non-NULL, where
    const float* r1_col;            // r1[m] = r1_row[m], or 0 when r1_gate is given and r1_gate[m] <= 0
    const float* r1_gate;
    float* r1_mask_colsum;          // += sum_m r1[m] * mask[m, n]   (the head's weight gradient)
    float* r1_sum;                  // += sum_m r1[m]                (the head's bias gradient)
    uint16_t* out;                  // [M, ld_out] in fmt
    int64_t ld_out;
    float* colsum;                  // += column sums of the stored values (a bias gradient) when non-NULL
    // Loss scale of a scaled backward: {scale, 1 / scale}.  The r1 term enters the
    // stored values multiplied by scale; colsum receives the sums times 1 / scale.
    // NULL = 1.  The head gradients (r1_mask_colsum, r1_sum) are never scaled.
    const float* gscale;
    int* found_inf;                 // set to 1 when a stored value is not finite or exceeds the fmt range
    // Head fused on the FP32 result rows: 1 (sigma), 3 (rgb) or 4 (sigma + rgb) dot products.
    int head_mode;
    const float* head_w;            // [units][N]
    const float* head_b;            // [units]
    const float* head_noise;        // [M] added to the raw sigma, or NULL
    float* head_sraw;               // [M] raw sigma
    float* head_sigma;              // [M] ReLU(raw sigma)
    float* head_rgb_ws;             // [M, 3] sigmoid rgb (kept for the backward)
    float* head_rgb_out;            // [M, 3] sigmoid rgb
    int* flag;
};

__host__ __device__ inline int head_units(int mode) {
    return mode == kHeadSigma ? 1 : (mode == kHeadRgb ? 3 : (mode == kHeadSigmaRgb ? 4 : 0));
}

// Epilogue features compiled into a kernel instance, as bit flags.  A launch takes
// the narrowest instantiated set that covers its GemmEpilogue: the branches of
// unused features, unrolled over every 32-column chunk, otherwise cost the 256-wide
// epilogue instruction fetch (measured: the forward layer ran 25% faster with them
// compiled out).  Always present: bias, ReLU, bits_out, found_inf, the output.
//   kEpiBits  mask_bits (the backward-data ReLU mask)
//   kEpiM16   the 16-bit mask
//   kEpiHead  the fused heads
//   kEpiR1    the r1 terms (r1_row / r1_col / r1_gate / r1_sum; r1_mask_colsum with kEpiM16)
//   kEpiCs    colsum
enum : int { kEpiFwd = 0, kEpiBits = 1, kEpiM16 = 2, kEpiHead = 4, kEpiR1 = 8, kEpiCs = 16, kEpiAll = 31 };

inline int epi_mode(const GemmEpilogue& ep) {
    int e = kEpiFwd;
    if (ep.mask_bits) e |= kEpiBits;
    if (ep.mask) e |= kEpiM16;
    if (head_units(ep.head_mode)) e |= kEpiHead;
    if (ep.r1_row || ep.r1_sum) e |= kEpiR1;
    if (ep.r1_mask_colsum) e |= kEpiM16 | kEpiR1;
    if (ep.colsum) e |= kEpiCs;
    return e;
}

// Lane i of the warp ends with sum over the 32 lanes of v[i] (recursive halving).
__device__ __forceinline__ float warp_reduce_scatter32(float (&v)[32]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int j = 0; j < off; ++j) {
            float send = upper ? v[j] : v[j + off];
            float keep = upper ? v[j + off] : v[j];
            v[j] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
    return v[0];
}

struct GemmShape {
    int64_t M;
    int kb0, kb1;   // 64-wide K blocks from A0 and A1
    int b_row0;     // first B row (output column 0)
};

// Output through TMA stores when every epilogue warp owns a multiple of 64 columns:
// each warp stages 32 rows x 64 columns (128-byte rows, 128-byte swizzle) and
// stores them with one bulk tensor copy.
constexpr bool tma_store_ok(int bn, int ew) { return (bn / (ew / 4)) % 64 == 0; }

template <int BN, int EW = 4>
struct SmemPlan {
    static constexpr uint32_t kBBlockBytes = BN * kBlockK * 2;
    static constexpr uint32_t kStoreBytes = tma_store_ok(BN, EW) ? uint32_t(EW) * 32 * 128 : 0u;
    // partial head sums handed between the two warps of a lane quadrant: [2 acc][128 rows][4]
    static constexpr uint32_t kHeadXBytes = EW == 8 ? 2 * 128 * 4 * 4 : 0u;
    // ReLU bits of one tile (forward, 4 epilogue warps): [4 warps][32 rows][BN / 32 words]
    static constexpr uint32_t kBitsBytes = EW == 4 ? 4u * 32 * (BN / 32) * 4 : 0u;
    // 1024 B alignment slack + 256 B of barriers + BN floats each of bias, column
    // sums and r1 mask column sums + 4 x BN head weights + 4 head biases + head exchange
    static constexpr size_t kReserve =
        1024 + 256 + BN * 12 + 4 * BN * 4 + 16 + kHeadXBytes + kStoreBytes + kBitsBytes;
    static __host__ __device__ int stages(int kb_total) {
        size_t b = size_t(kb_total) * kBBlockBytes;
        if (b + kReserve + 2 * kATileBytes > kMaxSmem) return 0;
        int s = int((kMaxSmem - kReserve - b) / kATileBytes);
        return s > 8 ? 8 : s;
    }
    static __host__ __device__ size_t bytes(int kb_total) {
        return kReserve + size_t(kb_total) * kBBlockBytes + size_t(stages(kb_total)) * kATileBytes;
    }
};

template <int BN, int EW, int EPI>
__global__ void __launch_bounds__(gemm_threads(EW), 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA0, const __grid_constant__ CUtensorMap tmA1,
                   const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmOut,
                   GemmShape shape, GemmEpilogue ep) {
    extern __shared__ uint8_t smem_raw[];
    // 1024-byte alignment for the swizzle atoms
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int kb_total = shape.kb0 + shape.kb1;
    using Plan = SmemPlan<BN, EW>;
    constexpr bool kTmaStore = tma_store_ok(BN, EW);
    const int stages = Plan::stages(kb_total);
    uint8_t* sB = base;
    uint8_t* sA = sB + size_t(kb_total) * Plan::kBBlockBytes;
    uint8_t* sOut = sA + size_t(stages) * kATileBytes;    // [EW warps][32 rows][128 B], 1024-aligned
    uint64_t* bars = reinterpret_cast<uint64_t*>(sOut + Plan::kStoreBytes);
    uint64_t* full = bars;              // [stages]
    uint64_t* empty = bars + 8;         // [stages]
    uint64_t* acc_full = bars + 16;     // [2]
    uint64_t* acc_empty = bars + 18;    // [2]
    uint64_t* b_full = bars + 20;
    uint64_t* done = bars + 21;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 22);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 23);
    uint64_t* hx_ready = bars + 24;     // [2 acc][4 quadrants]: half 1's partial head sums are in shx
    float* sbias = reinterpret_cast<float*>(bars + 32);   // BN floats
    float* scol = sbias + BN;                              // BN floats
    float* scol2 = scol + BN;                              // BN floats
    float* shw = scol2 + BN;                               // 4 x BN floats
    float* shb = shw + 4 * BN;                             // 4 floats
    float* shx = shb + 4;                                  // [2][128][4] partial head sums (8 epilogue warps)
    uint32_t* sbits = reinterpret_cast<uint32_t*>(shx + Plan::kHeadXBytes / 4);   // ReLU bits (4 epilogue warps)
    constexpr bool kBits = (EPI & kEpiBits) != 0, kM16 = (EPI & kEpiM16) != 0, kHd = (EPI & kEpiHead) != 0;
    constexpr bool kR1 = (EPI & kEpiR1) != 0, kCs = (EPI & kEpiCs) != 0;
    const int hunits = kHd ? head_units(ep.head_mode) : 0;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t num_tiles = (shape.M + kBlockM - 1) / kBlockM;

    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(&acc_full[a], 1);
            mbar_init(&acc_empty[a], 32 * EW);
        }
        mbar_init(b_full, 1);
        mbar_init(done, 1);
        for (int i = 0; i < 8; ++i) mbar_init(&hx_ready[i], 32);
        *abort_flag = 0;
        fence_barrier_init();
    }
    for (int i = threadIdx.x; i < BN; i += blockDim.x) {
        sbias[i] = ep.bias ? ep.bias[i] : 0.f;
        scol[i] = 0.f;
        scol2[i] = 0.f;
        for (int u = 0; u < hunits; ++u) shw[u * BN + i] = ep.head_w[u * BN + i];
    }
    if (threadIdx.x < 4) shb[threadIdx.x] = int(threadIdx.x) < hunits ? ep.head_b[threadIdx.x] : 0.f;
    if (warp == 1) {
        tmem_alloc(tmem_slot, 2 * BN);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---------------------------------------------------------- producer
        prefetch_tmap(&tmA0);
        if (shape.kb1) prefetch_tmap(&tmA1);
        prefetch_tmap(&tmB);
        if (kTmaStore) prefetch_tmap(&tmOut);
        mbar_arrive_expect_tx(b_full, uint32_t(kb_total) * Plan::kBBlockBytes);
        for (int kb = 0; kb < kb_total; ++kb)
            tma_load_2d(sB + size_t(kb) * Plan::kBBlockBytes, &tmB, b_full, kb * kBlockK, shape.b_row0);
        uint32_t it = 0;
        uint32_t last_parity[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        bool used[8] = {false, false, false, false, false, false, false, false};
        for (int64_t tile = blockIdx.x; tile < num_tiles && !*abort_flag; tile += gridDim.x) {
            for (int kb = 0; kb < kb_total; ++kb, ++it) {
                int s = int(it % stages);
                uint32_t ph = (it / stages) & 1;
                if (!mbar_wait(&empty[s], ph ^ 1, abort_flag)) {
                    *abort_flag = 1;
                    break;
                }
                mbar_arrive_expect_tx(&full[s], kATileBytes);
                int32_t row = int32_t(tile * kBlockM);
                if (kb < shape.kb0) tma_load_2d(sA + size_t(s) * kATileBytes, &tmA0, &full[s], kb * kBlockK, row);
                else tma_load_2d(sA + size_t(s) * kATileBytes, &tmA1, &full[s], (kb - shape.kb0) * kBlockK, row);
                used[s] = true;
                last_parity[s] = ph;
            }
        }
        // every copy this thread started has landed before the CTA may exit
        for (int s = 0; s < stages; ++s)
            if (used[s] && !mbar_wait(&full[s], last_parity[s], nullptr)) *abort_flag = 1;
        if (!mbar_wait(b_full, 0, nullptr)) *abort_flag = 1;
    } else if (warp == 1 && lane == 0) {
        // -------------------------------------------------------------- MMA
        const uint32_t idesc = idesc_f16(kBlockM, BN, 0, 0, ep.fmt);
        bool ok = mbar_wait(b_full, 0, abort_flag);
        uint32_t it = 0, t = 0;
        for (int64_t tile = blockIdx.x; ok && tile < num_tiles; tile += gridDim.x, ++t) {
            uint32_t acc = t & 1;
            if (!mbar_wait(&acc_empty[acc], ((t >> 1) & 1) ^ 1, abort_flag)) {
                ok = false;
                break;
            }
            tc_fence_after();
            uint32_t d_tmem = tmem + acc * BN;
            for (int kb = 0; kb < kb_total; ++kb, ++it) {
                int s = int(it % stages);
                if (!mbar_wait(&full[s], (it / stages) & 1, abort_flag)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                uint32_t a_addr = smem_u32(sA + size_t(s) * kATileBytes);
                uint32_t b_addr = smem_u32(sB + size_t(kb) * Plan::kBBlockBytes);
#pragma unroll
                for (int k = 0; k < kBlockK / 16; ++k) {
                    uint64_t ad = smem_desc(a_addr + k * 32, 0, 1024, kSwizzle128B);
                    uint64_t bd = smem_desc(b_addr + k * 32, 0, 1024, kSwizzle128B);
                    mma_f16(d_tmem, ad, bd, idesc, (kb | k) != 0);
                }
                mma_commit(&empty[s]);
            }
            if (!ok) break;
            mma_commit(&acc_full[acc]);
        }
        if (!ok) *abort_flag = 1;
        // all MMAs issued by this thread complete before tensor memory is freed
        mma_commit(done);
        if (!mbar_wait(done, 0, nullptr)) *abort_flag = 1;
    } else if (warp >= 2) {
        // --------------------------------------------------------- epilogue
        // Warp w reads the tensor-memory lane quadrant q = w % 4 (rows q*32 .. q*32+31
        // of the tile).  With 8 epilogue warps, w and w + 4 share a quadrant and `half`
        // 0 takes the first BN/2 columns, 1 the rest.
        static_assert(EW == 4 || EW == 8, "4 or 8 epilogue warps");
        const int q = warp & 3;
        const int half = EW == 8 ? (warp - 2) >> 2 : 0;
        constexpr int kHalfChunks = EW == 8 ? BN / 64 : BN / 32;   // 32-column chunks per warp
        const int c0 = half * kHalfChunks;
        uint32_t t = 0;
        float r1_total = 0.f;
        const float gs0 = ep.gscale ? ep.gscale[0] : 1.f;
        const float vmax = fmt_max(ep.fmt);
        bool bad = false;
        // 8 epilogue warps with mask bits: the row's words for this warp's chunks are
        // loaded before the accumulator wait, so their latency hides behind it
        constexpr bool kBitsAhead = kBits && EW == 8 && kHalfChunks <= 4;
        for (int64_t tile = blockIdx.x; tile < num_tiles; tile += gridDim.x, ++t) {
            uint32_t acc = t & 1;
            uint32_t mbw[kBitsAhead ? kHalfChunks : 1];
            if (kBitsAhead) {
                const int64_t mr = tile * kBlockM + q * 32 + lane;
                const uint32_t* src = ep.mask_bits + mr * ep.ld_bits + c0;
                if (kHalfChunks == 4 && (ep.ld_bits & 3) == 0) {   // one 16-byte load (c0 is 0 or 4)
                    const uint4 v = (ep.mask_bits && mr < shape.M) ? *reinterpret_cast<const uint4*>(src)
                                                                   : make_uint4(0u, 0u, 0u, 0u);
                    mbw[0] = v.x;
                    mbw[kHalfChunks > 1 ? 1 : 0] = v.y;
                    mbw[kHalfChunks > 2 ? 2 : 0] = v.z;
                    mbw[kHalfChunks > 3 ? 3 : 0] = v.w;
                } else {
#pragma unroll
                    for (int k = 0; k < (kBitsAhead ? kHalfChunks : 1); ++k)
                        mbw[k] = (ep.mask_bits && mr < shape.M) ? src[k] : 0u;
                }
            }
            if (!mbar_wait(&acc_full[acc], (t >> 1) & 1, abort_flag)) {
                *abort_flag = 1;
                break;
            }
            tc_fence_after();
            const int64_t m = tile * kBlockM + q * 32 + lane;
            const bool live = m < shape.M;
            float r1 = (kR1 && ep.r1_row && live) ? ep.r1_row[m] : 0.f;
            if (kR1 && ep.r1_gate && live && !(ep.r1_gate[m] > 0.f)) r1 = 0.f;
            if (half == 0) r1_total += r1;
            float hacc[4] = {0.f, 0.f, 0.f, 0.f};
            const uint32_t tbase = tmem + acc * BN + (uint32_t(q * 32) << 16);
            uint32_t rbuf[2][32];
            tmem_ld_32x32b_x32(tbase + uint32_t(c0 * 32), rbuf[0]);
            tmem_ld_wait();
            // chunks in pairs: the register buffer index stays static while only two copies
            // of the chunk body are inlined (8 warps: every chunk unrolled, at most 4, so
            // the ReLU bits of the row stay in registers)
            constexpr int kPairUnroll = EW == 8 ? (kHalfChunks + 1) / 2 : 1;
            uint32_t rbits[EW == 8 ? kHalfChunks : 1];
#pragma unroll kPairUnroll
            for (int cp = 0; cp < kHalfChunks; cp += 2)
#pragma unroll
            for (int hf = 0; hf < 2; ++hf) {
                const int cc = cp + hf;
                if (cc >= kHalfChunks) break;
                const int c = c0 + cc;
                uint32_t (&r)[32] = rbuf[hf];
                // start the next chunk's tensor-memory load; it completes under this chunk's math
                if (cc + 1 < kHalfChunks) tmem_ld_32x32b_x32(tbase + uint32_t((c + 1) * 32), rbuf[hf ^ 1]);
                float v[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    v[j] = __uint_as_float(r[j]) + sbias[c * 32 + j];
                    if (kR1 && ep.r1_row) v[j] += (r1 * gs0) * ep.r1_col[c * 32 + j];
                    if (ep.relu) v[j] = v[j] > 0.f ? v[j] : 0.f;
                    if (!live) v[j] = 0.f;
                }
                if (kBits && ep.mask_bits) {   // kernel-uniform branch
                    const uint32_t mb = kBitsAhead ? mbw[kBitsAhead ? cc : 0]
                                                   : (live ? ep.mask_bits[m * ep.ld_bits + c] : 0u);
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        if (!((mb >> j) & 1u)) v[j] = 0.f;
                }
                if (ep.bits_out) {   // stored after the tile's last chunk
                    uint32_t mb = 0u;
#pragma unroll
                    for (int j = 0; j < 32; ++j) mb |= uint32_t(v[j] > 0.f) << j;
                    if (EW == 8) rbits[cc] = mb;
                    else sbits[((warp - 2) * 32 + lane) * kHalfChunks + cc] = mb;
                }
                if (kM16 && ep.mask) {   // kernel-uniform branch; rows past M contribute zeros
                    float mw[32];
#pragma unroll
                    for (int j = 0; j < 32; ++j) mw[j] = 0.f;
                    if (live) {
                        const uint4* mp = reinterpret_cast<const uint4*>(ep.mask + m * ep.ld_mask + c * 32);
#pragma unroll
                        for (int g = 0; g < 4; ++g) {
                            uint4 mv = mp[g];
                            uint32_t w4[4] = {mv.x, mv.y, mv.z, mv.w};
#pragma unroll
                            for (int h = 0; h < 4; ++h) {
                                float2 f = unpack16(w4[h], ep.fmt);
                                mw[g * 8 + h * 2] = f.x;
                                mw[g * 8 + h * 2 + 1] = f.y;
                                if (!(f.x > 0.f)) v[g * 8 + h * 2] = 0.f;
                                if (!(f.y > 0.f)) v[g * 8 + h * 2 + 1] = 0.f;
                            }
                        }
                    }
                    if (kR1 && ep.r1_mask_colsum) {   // needs the mask; r1 is 0 on rows past M
#pragma unroll
                        for (int j = 0; j < 32; ++j) mw[j] *= r1;
                        atomicAdd(&scol2[c * 32 + lane], warp_reduce_scatter32(mw));
                    }
                }
                if (hunits) {
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        if (u < hunits) {
                            float sacc = 0.f;
#pragma unroll
                            for (int j = 0; j < 32; ++j) sacc += v[j] * shw[u * BN + c * 32 + j];
                            hacc[u] += sacc;
                        }
                    }
                }
                if (kTmaStore) {
                    // 16-byte piece jj of this lane's 128-byte row sits at jj ^ (row % 8) (the TMA
                    // 128-byte swizzle); rows past M are written but not stored (TMA clips them)
                    uint4* stg = reinterpret_cast<uint4*>(sOut) + (warp - 2) * 32 * 8 + lane * 8;
                    const int f = ep.fmt;
                    if ((cc & 1) == 0) {
                        // the previous 64-column store must have read the staging area
                        if (lane == 0) bulk_wait_read_all();
                        __syncwarp();
                    }
#pragma unroll
                    for (int g = 0; g < 4; ++g)
                        stg[(((cc & 1) * 4 + g) ^ (lane & 7))] =
                            make_uint4(pack16(v[g * 8], v[g * 8 + 1], f), pack16(v[g * 8 + 2], v[g * 8 + 3], f),
                                       pack16(v[g * 8 + 4], v[g * 8 + 5], f), pack16(v[g * 8 + 6], v[g * 8 + 7], f));
                    if (cc & 1) {
                        fence_proxy_async_smem();
                        __syncwarp();
                        if (lane == 0) {
                            tma_store_2d(&tmOut, stg, (c - 1) * 32, int32_t(tile * kBlockM + q * 32));
                            bulk_commit_group();
                        }
                    }
                    if (ep.found_inf && live) {
#pragma unroll
                        for (int j = 0; j < 32; ++j) bad |= !(fabsf(v[j]) <= vmax);
                    }
                } else if (live) {
                    uint4* op = reinterpret_cast<uint4*>(ep.out + m * ep.ld_out + c * 32);
                    const int f = ep.fmt;
#pragma unroll
                    for (int g = 0; g < 4; ++g)
                        op[g] = make_uint4(pack16(v[g * 8], v[g * 8 + 1], f), pack16(v[g * 8 + 2], v[g * 8 + 3], f),
                                           pack16(v[g * 8 + 4], v[g * 8 + 5], f),
                                           pack16(v[g * 8 + 6], v[g * 8 + 7], f));
                    if (ep.found_inf) {
#pragma unroll
                        for (int j = 0; j < 32; ++j) bad |= !(fabsf(v[j]) <= vmax);
                    }
                }
                if (kCs && ep.colsum) atomicAdd(&scol[c * 32 + lane], warp_reduce_scatter32(v));
                tmem_ld_wait();
            }
            if (EW == 4 && ep.bits_out) {
                // this warp's 32 rows x kHalfChunks words (whole rows: one warp covers BN)
                __syncwarp();
                const uint32_t* wb = sbits + (warp - 2) * 32 * kHalfChunks;
                if (ep.ld_bits == kHalfChunks && (kHalfChunks % 4) == 0) {
                    // the 32 rows are contiguous in bits_out: consecutive lanes store consecutive 16 bytes
                    const int64_t row0 = tile * kBlockM + q * 32;
                    uint4* dst = reinterpret_cast<uint4*>(ep.bits_out + row0 * ep.ld_bits);
                    const uint4* src = reinterpret_cast<const uint4*>(wb);
                    for (int i = lane; i < 32 * kHalfChunks / 4; i += 32)
                        if (row0 + (i * 4) / kHalfChunks < shape.M) dst[i] = src[i];
                } else if (live) {
                    for (int k = 0; k < kHalfChunks; ++k) ep.bits_out[m * ep.ld_bits + c0 + k] = wb[lane * kHalfChunks + k];
                }
                __syncwarp();
            }
            if (EW == 8 && ep.bits_out && live) {
                // this warp's kHalfChunks words of the row (words c0 .. c0 + kHalfChunks - 1)
                uint32_t* dst = ep.bits_out + m * ep.ld_bits + c0;
                if (kHalfChunks == 4 && (ep.ld_bits % 4) == 0) {
                    *reinterpret_cast<uint4*>(dst) = make_uint4(rbits[0], rbits[kHalfChunks > 1 ? 1 : 0],
                                                                rbits[kHalfChunks > 2 ? 2 : 0],
                                                                rbits[kHalfChunks > 3 ? 3 : 0]);
                } else {
#pragma unroll
                    for (int k = 0; k < kHalfChunks; ++k) dst[k] = rbits[k];
                }
            }
            if (EW == 8 && hunits) {   // kernel-uniform: half 1 hands its partial dot products to half 0
                // The slot of accumulator `acc` is rewritten two tiles later, only after this
                // tile's acc_empty completed, which needs half 0's arrival below: no reuse race.
                float* x = shx + (acc * 128 + q * 32 + lane) * 4;
                uint64_t* rdy = &hx_ready[acc * 4 + q];
                if (half == 1) {
#pragma unroll
                    for (int u = 0; u < 4; ++u) x[u] = hacc[u];
                    mbar_arrive(rdy);
                } else if (mbar_wait(rdy, (t >> 1) & 1, abort_flag)) {
#pragma unroll
                    for (int u = 0; u < 4; ++u) hacc[u] += x[u];
                } else {
                    *abort_flag = 1;
                }
            }
            if (hunits && live && half == 0) {
                // SimpleNeRF17.py:735-750 (sigma head + noise + ReLU) and :771-777 (sigmoid rgb)
                int u0 = 0;
                if (ep.head_mode != kHeadRgb) {
                    float s = hacc[0] + shb[0];
                    if (ep.head_noise) s += ep.head_noise[m];
                    ep.head_sraw[m] = s;
                    ep.head_sigma[m] = s > 0.f ? s : 0.f;
                    u0 = 1;
                }
                if (ep.head_mode != kHeadSigma) {
#pragma unroll
                    for (int cc = 0; cc < 3; ++cc) {
                        float rv = 1.f / (1.f + expf(-(hacc[u0 + cc] + shb[u0 + cc])));
                        ep.head_rgb_ws[3 * m + cc] = rv;
                        ep.head_rgb_out[3 * m + cc] = rv;
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(&acc_empty[acc]);
        }
        if (kR1 && ep.r1_sum) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) r1_total += __shfl_xor_sync(0xffffffffu, r1_total, o);
            if (lane == 0) atomicAdd(ep.r1_sum, r1_total);
        }
        if (ep.found_inf && __any_sync(0xffffffffu, bad) && lane == 0) atomicExch(ep.found_inf, 1);
        // every bulk store of this warp has completed before the CTA may exit
        if (kTmaStore && lane == 0) bulk_wait_all();
    }
    __syncthreads();
    if (threadIdx.x == 0 && *abort_flag) raise_flag(ep.flag, kFlagTimeout);
    if (kCs && ep.colsum) {
        const float gs1 = ep.gscale ? ep.gscale[1] : 1.f;
        for (int i = threadIdx.x; i < BN; i += blockDim.x) atomicAdd(ep.colsum + i, scol[i] * gs1);
    }
    if (kM16 && kR1 && ep.r1_mask_colsum)
        for (int i = threadIdx.x; i < BN; i += blockDim.x) atomicAdd(ep.r1_mask_colsum + i, scol2[i]);
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 2 * BN);
    }
}

// --------------------------------------------------------------------------
// Weight gradient: partial[split, n, k] = sum_{m in split} dZ[m, n] * X[m, k]
// for one 128-row block of n and all k (X = [X0 | X1], at most 512 columns).
// The reduction runs over samples, so both operands are MN-major in shared
// memory: TMA boxes of 64 samples x 64 features (128-byte swizzle), LBO = the
// 8 KB step between 64-wide feature chunks, SBO = 1024 B between 8-sample groups.
// --------------------------------------------------------------------------

struct WgradShape {
    int64_t M;        // samples
    int64_t m_chunk;  // samples per split (multiple of 64)
    int n_dz;         // columns of dZ (rows of dW)
    int kc0, kc1;     // 64-wide column chunks of X0 / X1
    int fmt;          // operand format (kFmtBF16, kFmtF16)
    int ones;         // also sum dZ over the samples (a bias gradient), added into bias_grad
};

constexpr uint32_t kBox64Bytes = 64 * 64 * 2;

// A stage holds the two dZ boxes and the X boxes of 64 samples; one more box of
// 16-bit ones (when the bias gradient is wanted) is an MMA operand whose product
// with dZ^T is the sum of dZ over the samples.
__host__ __device__ inline int wgrad_stages(int nchunks, int ones) {
    size_t stage = size_t(2 + nchunks) * kBox64Bytes;
    int s = int((kMaxSmem - 1024 - 256 - (ones ? kBox64Bytes : 0)) / stage);
    return s > 6 ? 6 : s;
}
__host__ __device__ inline size_t wgrad_smem(int nchunks, int ones) {
    return 1024 + 256 + size_t(wgrad_stages(nchunks, ones)) * (2 + nchunks) * kBox64Bytes +
           (ones ? kBox64Bytes : 0);
}
__host__ __device__ inline uint32_t tmem_cols_for(int n) {
    uint32_t c = 32;
    while (c < uint32_t(n)) c <<= 1;
    return c;
}

__global__ void __launch_bounds__(kThreads, 1)
    tc_wgrad_kernel(const __grid_constant__ CUtensorMap tmDZ, const __grid_constant__ CUtensorMap tmX0,
                    const __grid_constant__ CUtensorMap tmX1, WgradShape s, float* partial, float* bias_grad,
                    const float* gscale, int* flag) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int nchunks = s.kc0 + s.kc1;
    const int np = nchunks * 64;
    const int stages = wgrad_stages(nchunks, s.ones);
    const uint32_t stage_bytes = uint32_t(2 + nchunks) * kBox64Bytes;
    uint8_t* sones = base + size_t(stages) * stage_bytes;   // 1024-aligned (stage_bytes is a multiple of 8 KB)
    uint64_t* bars = reinterpret_cast<uint64_t*>(sones + (s.ones ? kBox64Bytes : 0));
    uint64_t* full = bars;
    uint64_t* empty = bars + 8;
    uint64_t* acc_full = bars + 16;
    uint64_t* done = bars + 17;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 18);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 19);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.x * 128;
    const int64_t m_begin = int64_t(blockIdx.y) * s.m_chunk;
    int64_t m_end = m_begin + s.m_chunk;
    if (m_end > s.M) m_end = s.M;
    const int nblk = m_end > m_begin ? int((m_end - m_begin + 63) / 64) : 0;
    const uint32_t ncols = tmem_cols_for(np + (s.ones ? 64 : 0));
    if (s.ones) {   // 16-bit ones for the generic proxy, then made visible to the tensor core
        const uint32_t one2 = s.fmt == kFmtF16 ? 0x3C003C00u : 0x3F803F80u;
        uint4* o = reinterpret_cast<uint4*>(sones);
        for (int i = threadIdx.x; i < int(kBox64Bytes / 16); i += blockDim.x) o[i] = make_uint4(one2, one2, one2, one2);
        fence_proxy_async_smem();
    }

    if (threadIdx.x == 0) {
        for (int i = 0; i < stages; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        mbar_init(acc_full, 1);
        mbar_init(done, 1);
        *abort_flag = 0;
        fence_barrier_init();
    }
    if (warp == 1) {
        tmem_alloc(tmem_slot, ncols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        prefetch_tmap(&tmDZ);
        prefetch_tmap(&tmX0);
        if (s.kc1) prefetch_tmap(&tmX1);
        uint32_t last_parity[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        bool used[8] = {false, false, false, false, false, false, false, false};
        for (int b = 0; b < nblk; ++b) {
            int st = b % stages;
            uint32_t ph = (b / stages) & 1;
            if (!mbar_wait(&empty[st], ph ^ 1, abort_flag)) {
                *abort_flag = 1;
                break;
            }
            uint8_t* sa = base + size_t(st) * stage_bytes;
            int32_t row = int32_t(m_begin + int64_t(b) * 64);
            mbar_arrive_expect_tx(&full[st], stage_bytes);
            tma_load_2d(sa, &tmDZ, &full[st], n0, row);
            tma_load_2d(sa + kBox64Bytes, &tmDZ, &full[st], n0 + 64, row);
            for (int c = 0; c < nchunks; ++c) {
                uint8_t* dst = sa + size_t(2 + c) * kBox64Bytes;
                if (c < s.kc0) tma_load_2d(dst, &tmX0, &full[st], c * 64, row);
                else tma_load_2d(dst, &tmX1, &full[st], (c - s.kc0) * 64, row);
            }
            used[st] = true;
            last_parity[st] = ph;
        }
        for (int i = 0; i < stages; ++i)
            if (used[i] && !mbar_wait(&full[i], last_parity[i], nullptr)) *abort_flag = 1;
    } else if (warp == 1 && lane == 0) {
        bool ok = true;
        for (int b = 0; b < nblk; ++b) {
            int st = b % stages;
            if (!mbar_wait(&full[st], (b / stages) & 1, abort_flag)) {
                ok = false;
                break;
            }
            tc_fence_after();
            uint32_t sa = smem_u32(base + size_t(st) * stage_bytes);
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
                uint64_t ad = smem_desc(sa + ks * 2048, kBox64Bytes, 1024, kSwizzle128B);
                for (int p = 0; p * 4 < nchunks; ++p) {
                    int cnt = nchunks - p * 4 < 4 ? nchunks - p * 4 : 4;
                    uint64_t bd = smem_desc(sa + (2 + p * 4) * kBox64Bytes + ks * 2048, kBox64Bytes, 1024,
                                            kSwizzle128B);
                    mma_f16(tmem + uint32_t(p * 256), ad, bd, idesc_f16(128, cnt * 64, 1, 1, s.fmt),
                             (b | ks) != 0);
                }
                if (s.ones) {   // columns np .. np + 63: every one is sum_m dz[m, n]
                    uint64_t od = smem_desc(smem_u32(sones) + ks * 2048, kBox64Bytes, 1024, kSwizzle128B);
                    mma_f16(tmem + uint32_t(np), ad, od, idesc_f16(128, 64, 1, 1, s.fmt), (b | ks) != 0);
                }
            }
            mma_commit(&empty[st]);
        }
        if (!ok) *abort_flag = 1;
        mma_commit(acc_full);
        mma_commit(done);
        if (!mbar_wait(done, 0, nullptr)) *abort_flag = 1;
    } else if (warp >= 2) {
        const int q = warp & 3;
        bool ok = mbar_wait(acc_full, 0, abort_flag);
        if (!ok) *abort_flag = 1;
        tc_fence_after();
        const int n = n0 + q * 32 + lane;
        float* dst = partial + (int64_t(blockIdx.y) * s.n_dz + n) * np;
        for (int c = 0; c < np / 32; ++c) {
            uint32_t r[32];
            tmem_ld_32x32b_x32(tmem + (uint32_t(q * 32) << 16) + uint32_t(c * 32), r);
            tmem_ld_wait();
            if (n >= s.n_dz) continue;
            float4* o = reinterpret_cast<float4*>(dst + c * 32);
#pragma unroll
            for (int g = 0; g < 8; ++g) {
                float4 v;
                if (nblk > 0 && ok) {
                    v = make_float4(__uint_as_float(r[4 * g]), __uint_as_float(r[4 * g + 1]),
                                    __uint_as_float(r[4 * g + 2]), __uint_as_float(r[4 * g + 3]));
                } else {
                    v = make_float4(0.f, 0.f, 0.f, 0.f);
                }
                o[g] = v;
            }
        }
        if (s.ones) {
            uint32_t r[32];
            tmem_ld_32x32b_x32(tmem + (uint32_t(q * 32) << 16) + uint32_t(np), r);
            tmem_ld_wait();
            // this split's part, times 1 / loss scale; one atomic per dZ column and split
            if (n < s.n_dz && nblk > 0 && ok) atomicAdd(bias_grad + n, __uint_as_float(r[0]) * (gscale ? gscale[1] : 1.f));
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && *abort_flag) raise_flag(flag, kFlagTimeout);
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, ncols);
    }
}

}  // namespace tc
}  // namespace srf
