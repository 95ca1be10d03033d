// 16-bit tensor-core (tcgen05) path of the NeRF MLP: FP32 master weights, BF16
// or FP16 operands (weights and activations in HBM), FP32 accumulation in tensor
// memory.  The FP16 format keeps 3 more mantissa bits; its backward runs on
// loss-scaled gradients (srf_loss_scaler) so they stay in range.  PE sin/cos is
// computed in FP32; the small heads (sigma: 1 output, rgb: 3 outputs) are FP32
// dot products fused into the epilogue of the layer that feeds them.
//
// Forward per layer: one persistent tcgen05 GEMM with the bias/ReLU epilogue.
// Backward per layer: a dgrad GEMM (dZ . W^T with the ReLU mask of the forward
// activation and the bias gradient fused into its epilogue) and a split-K wgrad
// GEMM over samples (MN-major operands) reduced into the FP32 weight gradient.
#include <cudaTypedefs.h>

#include <atomic>
#include <cstring>
#include <mutex>
#include <vector>

#include "nerf_mlp.h"

#include "autotune.cuh"
#include "tc_gemm.cuh"
#include "tc_mlp_fused.cuh"

namespace srf {

using op16 = uint16_t;   // one 16-bit operand word: BF16 or FP16 bits, by the path's format

namespace {

// ----------------------------------------------------------- tensor maps ---

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        cudaGetLastError();
    });
    return fn;
}

// 2-D BF16 map: `inner` contiguous elements per row, `outer` rows of `row_bytes`.
bool make_map(CUtensorMap* m, const void* ptr, uint64_t inner, uint64_t outer, uint64_t row_bytes, uint32_t box_in,
              uint32_t box_out) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {row_bytes};
    cuuint32_t box[2] = {box_in, box_out};
    cuuint32_t es[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int num_sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
    }
    return n;
}

bool ok16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

template <int BN, int EW, int EPI>
int launch_gemm_epi(const CUtensorMap& a0, const CUtensorMap& a1, const CUtensorMap& b, const CUtensorMap& out,
                    tc::GemmShape sh, tc::GemmEpilogue ep, size_t smem, cudaStream_t s) {
    static bool attr_done = false;
    if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(tc::tc_gemm_kernel<BN, EW, EPI>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, int(tc::kMaxSmem));
        if (e != cudaSuccess) {
            set_cuda_error(e);
            return SRF_ERR_CUDA;
        }
        attr_done = true;
    }
    int64_t tiles = (sh.M + tc::kBlockM - 1) / tc::kBlockM;
    int grid = int(tiles < num_sms() ? tiles : num_sms());
    tc::tc_gemm_kernel<BN, EW, EPI><<<grid, tc::gemm_threads(EW), smem, s>>>(a0, a1, b, out, sh, ep);
    return launch_status();
}

template <int BN, int EW>
int launch_gemm_ew(const CUtensorMap& a0, const CUtensorMap& a1, const CUtensorMap& b, const CUtensorMap& out,
                   tc::GemmShape sh, tc::GemmEpilogue ep, cudaStream_t s) {
    int kb = sh.kb0 + sh.kb1;
    if (tc::SmemPlan<BN, EW>::stages(kb) < 2) return SRF_ERR_UNSUPPORTED;
    size_t smem = tc::SmemPlan<BN, EW>::bytes(kb);
    switch (tc::epi_mode(ep)) {   // the combinations the layers use; anything else runs the full set
        case tc::kEpiFwd: return launch_gemm_epi<BN, EW, tc::kEpiFwd>(a0, a1, b, out, sh, ep, smem, s);
        case tc::kEpiBits: return launch_gemm_epi<BN, EW, tc::kEpiBits>(a0, a1, b, out, sh, ep, smem, s);
        case tc::kEpiBits | tc::kEpiR1:
            return launch_gemm_epi<BN, EW, tc::kEpiBits | tc::kEpiR1>(a0, a1, b, out, sh, ep, smem, s);
        case tc::kEpiM16: return launch_gemm_epi<BN, EW, tc::kEpiM16>(a0, a1, b, out, sh, ep, smem, s);
        case tc::kEpiHead: return launch_gemm_epi<BN, EW, tc::kEpiHead>(a0, a1, b, out, sh, ep, smem, s);
        default: return launch_gemm_epi<BN, EW, tc::kEpiAll>(a0, a1, b, out, sh, ep, smem, s);
    }
}

// 8 epilogue warps (two per tensor-memory lane quadrant) keep the TMA-store epilogue
// ahead of the memory system; they need two more 4 KB staging areas, so layers whose
// resident weights leave fewer than two activation stages (K = 320 at N = 256) and the
// 64-wide layers (32 columns per warp: no 64-column TMA boxes) run on 4.
// Where both fit and the epilogue only overwrites its outputs, the tuner times the two
// on the first call of each (BN, K blocks, epilogue flags) and keeps the faster.
template <int BN>
int launch_gemm_bn(const CUtensorMap& a0, const CUtensorMap& a1, const CUtensorMap& b, const CUtensorMap& out,
                   tc::GemmShape sh, tc::GemmEpilogue ep, cudaStream_t s) {
    const int kb = sh.kb0 + sh.kb1;
    const bool eight = BN >= 128 && tc::SmemPlan<BN, 8>::stages(kb) >= 2;
    const bool four = tc::SmemPlan<BN, 4>::stages(kb) >= 2;
    const bool pure = !ep.colsum && !ep.r1_sum && !ep.r1_mask_colsum;
    auto run = [&](int i) {
        return i == 0 ? launch_gemm_ew<BN, 8>(a0, a1, b, out, sh, ep, s) : launch_gemm_ew<BN, 4>(a0, a1, b, out, sh, ep, s);
    };
    if (eight && four && pure) {
        const tune::Key key{tune::kSiteGemmEpilogueWarps, BN, kb, tc::epi_mode(ep)};
        return run(tune::pick(key, 2, 0, s, run));
    }
    return run(eight ? 0 : 1);
}

}  // namespace

tc::GemmEpilogue make_epilogue(op16* out, int64_t ld_out, const float* bias, int relu, int fmt = tc::kFmtBF16,
                               int* found_inf = nullptr) {
    tc::GemmEpilogue ep{};
    ep.fmt = fmt;
    ep.found_inf = found_inf;
    ep.out = out;
    ep.ld_out = ld_out;
    ep.bias = bias;
    ep.relu = relu;
    ep.head_mode = tc::kHeadNone;
    ep.flag = device_flag();
    return ep;
}

// ep.out[m, :n] = epilogue(x0[m, :k0] . B0^T + x1[m, :k1] . B1^T) with B the rows
// [w_row0, w_row0 + n) of the BF16 matrix w (w_rows x ldw, K-major).
int tc_linear(const tc::GemmEpilogue& ep, const op16* x0, int64_t ld0, int k0, const op16* x1, int64_t ld1, int k1,
              const op16* w, int64_t ldw, int w_rows, int w_row0, int64_t M, int n, cudaStream_t s) {
    const op16* mask = ep.mask;
    const int64_t ld_out = ep.ld_out, ld_mask = ep.ld_mask;
    if (M <= 0) return SRF_OK;
    if (!ep.out || !x0 || !w) return SRF_ERR_NULL;
    if (ep.head_mode && (!ep.head_w || !ep.head_b)) return SRF_ERR_NULL;
    if (ep.r1_mask_colsum && !mask) return SRF_ERR_NULL;
    if ((k0 % 64) || (k1 % 64) || k0 <= 0 || (k1 && !x1)) return SRF_ERR_SHAPE;
    if (n != 64 && n != 128 && n != 256) return SRF_ERR_UNSUPPORTED;
    if (w_row0 < 0 || w_row0 + n > w_rows || ldw < k0 + k1) return SRF_ERR_SHAPE;
    if (ld_out < n || ld0 < k0 || (x1 && ld1 < k1) || (mask && ld_mask < n)) return SRF_ERR_SHAPE;
    if (!ok16(ep.out) || !ok16(x0) || !ok16(w) || (x1 && !ok16(x1)) || (mask && !ok16(mask))) return SRF_ERR_ALIGN;
    if ((ld_out % 8) || (ld0 % 8) || (ldw % 8) || (x1 && (ld1 % 8)) || (mask && (ld_mask % 8))) return SRF_ERR_ALIGN;
    CUtensorMap ma0, ma1, mb;
    if (!make_map(&ma0, x0, uint64_t(k0), uint64_t(M), uint64_t(ld0) * 2, 64, tc::kBlockM)) return SRF_ERR_CUDA;
    if (x1) {
        if (!make_map(&ma1, x1, uint64_t(k1), uint64_t(M), uint64_t(ld1) * 2, 64, tc::kBlockM)) return SRF_ERR_CUDA;
    } else {
        ma1 = ma0;
    }
    if (!make_map(&mb, w, uint64_t(k0 + k1), uint64_t(w_rows), uint64_t(ldw) * 2, 64, uint32_t(n)))
        return SRF_ERR_CUDA;
    // output map for the TMA-store epilogue: n columns of rows ld_out apart, 64 x 32 boxes
    CUtensorMap mo;
    if (!make_map(&mo, ep.out, uint64_t(n), uint64_t(M), uint64_t(ld_out) * 2, 64, 32)) return SRF_ERR_CUDA;
    tc::GemmShape sh{M, k0 / 64, k1 / 64, w_row0};
    switch (n) {
        case 64: return launch_gemm_bn<64>(ma0, ma1, mb, mo, sh, ep, s);
        case 128: return launch_gemm_bn<128>(ma0, ma1, mb, mo, sh, ep, s);
        default: return launch_gemm_bn<256>(ma0, ma1, mb, mo, sh, ep, s);
    }
}

// splits <= num_sms / (n_dz / 128), so splits * n_dz <= num_sms * 128
size_t tc_wgrad_partial_floats(int n_dz, int np) {
    (void)n_dz;
    return size_t(num_sms()) * 128 * np;
}

// partial[split, n, k] = sum_m dz[m, n] x[m, k] (x = [x0 | x1]); returns the split count.
int tc_wgrad(float* partial, size_t partial_floats, const op16* dz, int64_t ld_dz, int n_dz, const op16* x0,
             int64_t ld0, int k0, const op16* x1, int64_t ld1, int k1, int64_t M, int* splits_out, cudaStream_t s,
             int fmt = tc::kFmtBF16, float* bias_grad = nullptr, const float* gscale = nullptr) {
    const bool ones = bias_grad != nullptr;
    if (n_dz % 128 || k0 % 64 || k1 % 64 || k0 <= 0 || k0 + k1 > (ones ? 448 : 512)) return SRF_ERR_UNSUPPORTED;
    if (ld_dz < n_dz || ld0 < k0 || (k1 && (!x1 || ld1 < k1))) return SRF_ERR_SHAPE;
    if (!ok16(dz) || !ok16(x0) || (x1 && !ok16(x1)) || (ld_dz % 8) || (ld0 % 8) || (x1 && (ld1 % 8)))
        return SRF_ERR_ALIGN;
    int ntile = n_dz / 128;
    int splits = num_sms() / ntile;
    if (splits < 1) splits = 1;
    int64_t blocks = (M + 63) / 64;
    if (splits > blocks) splits = int(blocks > 0 ? blocks : 1);
    int64_t chunk = ((blocks + splits - 1) / splits) * 64;
    splits = int((M + chunk - 1) / chunk);
    if (splits < 1) splits = 1;
    int np = k0 + k1;
    if (size_t(splits) * n_dz * np > partial_floats) return SRF_ERR_WORKSPACE;
    CUtensorMap mdz, m0, m1;
    if (!make_map(&mdz, dz, uint64_t(n_dz), uint64_t(M), uint64_t(ld_dz) * 2, 64, 64)) return SRF_ERR_CUDA;
    if (!make_map(&m0, x0, uint64_t(k0), uint64_t(M), uint64_t(ld0) * 2, 64, 64)) return SRF_ERR_CUDA;
    if (x1) {
        if (!make_map(&m1, x1, uint64_t(k1), uint64_t(M), uint64_t(ld1) * 2, 64, 64)) return SRF_ERR_CUDA;
    } else {
        m1 = m0;
    }
    int nchunks = np / 64;
    if (tc::wgrad_stages(nchunks, ones) < 2) return SRF_ERR_UNSUPPORTED;
    static bool attr_done = false;
    if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(tc::tc_wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(tc::kMaxSmem));
        if (e != cudaSuccess) {
            set_cuda_error(e);
            return SRF_ERR_CUDA;
        }
        attr_done = true;
    }
    tc::WgradShape sh{M, chunk, n_dz, k0 / 64, k1 / 64, fmt, ones ? 1 : 0};
    dim3 grid(ntile, splits);
    tc::tc_wgrad_kernel<<<grid, tc::kThreads, tc::wgrad_smem(nchunks, ones), s>>>(mdz, m0, m1, sh, partial,
                                                                                bias_grad, gscale, device_flag());
    *splits_out = splits;
    return launch_status();
}

namespace {

// ----------------------------------------------------------- small kernels --

// One layer's padded BF16 weight layout: up to two K sources; source i covers
// padded columns [pad0_i, pad0_i + padw_i) holding reference columns
// [ref0_i, ref0_i + refw_i) (the rest zero).
struct LayerMap {
    int n;
    int nsrc;
    int pad0[2], padw[2], ref0[2], refw[2];
    // Blocked first source (nblk > 0): its first nblk blocks of bwr reference columns
    // each sit at padded stride bwp (bwp - bwr zero columns after each block), the
    // rest of the source follows from padded column nblk * bwp.
    int nblk, bwp, bwr;
    __host__ __device__ int kpad() const { return pad0[nsrc - 1] + padw[nsrc - 1]; }
    __host__ __device__ int kref() const { return ref0[nsrc - 1] + refw[nsrc - 1]; }
};

__device__ __forceinline__ int ref_col(const LayerMap& L, int kp) {
    for (int i = 0; i < L.nsrc; ++i) {
        int off = kp - L.pad0[i];
        if (off >= 0 && off < L.padw[i]) {
            if (i == 0 && L.nblk > 0) {
                const int head = L.nblk * L.bwp;
                if (off < head) {
                    const int b = off / L.bwp, j = off - b * L.bwp;
                    return j < L.bwr ? L.ref0[0] + b * L.bwr + j : -1;
                }
                const int r = L.nblk * L.bwr + (off - head);
                return r < L.refw[0] ? L.ref0[0] + r : -1;
            }
            return off < L.refw[i] ? L.ref0[i] + off : -1;
        }
    }
    return -1;
}

// W (n x kref, fp32) -> Wp (n x kpad) and WT (kpad x n), 16-bit words of format fmt.
__global__ void pack_weight_kernel(LayerMap L, const float* __restrict__ w, op16* wp, op16* wt, int fmt) {
    int kp = blockIdx.x * blockDim.x + threadIdx.x;
    int n = blockIdx.y;
    int kpad = L.kpad();
    if (kp >= kpad) return;
    int rc = ref_col(L, kp);
    float v = rc >= 0 ? w[int64_t(n) * L.kref() + rc] : 0.f;
    op16 b = tc::to16(v, fmt);
    wp[int64_t(n) * kpad + kp] = b;
    wt[int64_t(kp) * L.n + n] = b;
}

// Up to kPackBatch layers' W -> (Wp, WT) in one launch (blockIdx.z = layer).
constexpr int kPackBatch = 12;
struct PackBatch {
    LayerMap lm[kPackBatch];
    const float* w[kPackBatch];
    op16* wp[kPackBatch];
    op16* wt[kPackBatch];
};

__global__ void pack_weights_kernel(const __grid_constant__ PackBatch b, int fmt) {
    const LayerMap& L = b.lm[blockIdx.z];
    const int kp = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = blockIdx.y;
    const int kpad = L.kpad();
    if (kp >= kpad || n >= L.n) return;
    const int rc = ref_col(L, kp);
    const float v = rc >= 0 ? b.w[blockIdx.z][int64_t(n) * L.kref() + rc] : 0.f;
    const op16 h = tc::to16(v, fmt);
    b.wp[blockIdx.z][int64_t(n) * kpad + kp] = h;
    b.wt[blockIdx.z][int64_t(kp) * L.n + n] = h;
}

// grad[n, ref] += sum_s partial[s, n, kp] (times 1 / loss scale when gscale) for the mapped columns.
// A block covers 128 columns of one row n: lane j of warp w adds the 16-byte column
// quads 4j .. 4j + 3 of splits w, w + 4, ... (512 coalesced bytes a warp load), and the
// four partial sums meet in shared memory (the same order of additions per column as
// one column per lane).  kpad is a multiple of 64, so a quad is whole or absent.
__global__ void __launch_bounds__(128) reduce_wgrad_kernel(LayerMap L, const float* __restrict__ partial, int splits,
                                                           int n_dz, float* grad, const float* gscale) {
    __shared__ float4 part[4][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int kp = blockIdx.x * 128 + lane * 4;
    const int n = blockIdx.y;
    const int kpad = L.kpad();
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    if (kp < kpad) {
        const float4* src = reinterpret_cast<const float4*>(partial + int64_t(n) * kpad + kp);
        const int64_t step = int64_t(n_dz) * kpad / 4;
#pragma unroll 4
        for (int sp = warp; sp < splits; sp += 4) {
            const float4 v = src[sp * step];
            acc.x += v.x;
            acc.y += v.y;
            acc.z += v.z;
            acc.w += v.w;
        }
    }
    part[warp][lane] = acc;
    __syncthreads();
    if (warp == 0 && kp < kpad) {
        const float4 a = part[0][lane], b = part[1][lane], c = part[2][lane], d = part[3][lane];
        const float sums[4] = {a.x + b.x + c.x + d.x, a.y + b.y + c.y + d.y, a.z + b.z + c.z + d.z,
                               a.w + b.w + c.w + d.w};
        const float gs = gscale ? gscale[1] : 1.f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int rc = ref_col(L, kp + q);
            if (rc >= 0) grad[int64_t(n) * L.kref() + rc] += gscale ? sums[q] * gs : sums[q];
        }
    }
}

// enc[m] = PE(pts[m], Lp)[:pin] zero-padded to enc_w; vext[m] = [PE(pts[m])[pin:ppe],
// PE(dirs[m/div], Lv)] zero-padded to vx_w, in format fmt, with PE(x, L) = [x,
// sin(2^0 x), cos(2^0 x), ..., sin(2^(L-1) x), cos(2^(L-1) x)] in 3-wide blocks
// (SimpleNeRF17.py:581-613).  One thread builds one row in shared memory (one
// sincosf per frequency and axis); the block then stores its kEncRows rows with
// consecutive threads on consecutive 4-byte words.  The row stride of
// enc_w + vx_w + 2 words16 (an odd number of 4-byte words) keeps the per-row
// writes free of bank conflicts.
constexpr int kEncRows = 64;

__global__ void __launch_bounds__(kEncRows)
    encode16_kernel(const float* __restrict__ pts, const float* __restrict__ dirs, int div, int64_t M, int lp,
                    int lv, int pin, int enc_w, int vx_w, op16* enc, op16* vext, int fmt) {
    extern __shared__ uint32_t enc_smem[];
    const int stride = enc_w + vx_w + 2;   // 16-bit words per staged row
    op16* srow = reinterpret_cast<op16*>(enc_smem);
    const int64_t row0 = int64_t(blockIdx.x) * kEncRows;
    const int r = threadIdx.x;
    const int64_t m = row0 + r;
    op16* my = srow + r * stride;
    for (int c = 0; c < (enc_w + vx_w) / 2; ++c) reinterpret_cast<uint32_t*>(my)[c] = 0u;
    if (m < M) {
        const int ppe = 3 * (2 * lp + 1);
        const float p[3] = {pts[3 * m], pts[3 * m + 1], pts[3 * m + 2]};
        // column col of PE(pts): enc below pin, the rest continues vext (dropped when there is none)
        auto put = [&](int col, float v) {
            if (col < pin) my[col] = tc::to16(v, fmt);
            else if (col - pin < vx_w) my[enc_w + (col - pin)] = tc::to16(v, fmt);
        };
#pragma unroll
        for (int a = 0; a < 3; ++a) put(a, p[a]);
        for (int k = 0; k < lp; ++k) {
            const float f = float(1 << k);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                float sn, cs;
                sincosf(p[a] * f, &sn, &cs);
                put(3 + 6 * k + a, sn);
                put(6 + 6 * k + a, cs);
            }
        }
        if (dirs && vext && (ppe - pin) + 3 * (2 * lv + 1) <= vx_w) {
            const float* d = dirs + 3 * (m / div);
            const float q[3] = {d[0], d[1], d[2]};
            op16* vd = my + enc_w + (ppe - pin);
#pragma unroll
            for (int a = 0; a < 3; ++a) vd[a] = tc::to16(q[a], fmt);
            for (int k = 0; k < lv; ++k) {
                const float f = float(1 << k);
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    float sn, cs;
                    sincosf(q[a] * f, &sn, &cs);
                    vd[3 + 6 * k + a] = tc::to16(sn, fmt);
                    vd[6 + 6 * k + a] = tc::to16(cs, fmt);
                }
            }
        }
    }
    __syncthreads();
    const int64_t rows = M - row0 < kEncRows ? M - row0 : kEncRows;
    const uint32_t* src = enc_smem;
    const int we = enc_w / 2, wv = vx_w / 2, ws = stride / 2;
    uint32_t* ge = reinterpret_cast<uint32_t*>(enc + row0 * enc_w);
    for (int w = threadIdx.x; w < rows * we; w += kEncRows) ge[w] = src[(w / we) * ws + w % we];
    if (vext) {
        uint32_t* gv = reinterpret_cast<uint32_t*>(vext + row0 * vx_w);
        for (int w = threadIdx.x; w < rows * wv; w += kEncRows) gv[w] = src[(w / wv) * ws + we + w % wv];
    }
}

// Backward of a small head (1-4 outputs) fused with what consumes it, in one
// pass over the head's input activation h (16-bit format fmt, M x K):
//   g[m]       = head output gradients (mode 3: rgb; mode 4: sigma + rgb), through
//                the ReLU of the raw sigma and the sigmoid of rgb;
//   dz[m, k]   = S (sum_u g[m, u] W[u, k]) * (h[m, k] > 0)   (fmt, the previous layer's dZ,
//                times the loss scale S = gscale[0], 1 when gscale is NULL)
//   colsum[k] += sum_m dz[m, k] / S                          (that layer's bias gradient, when given)
//   dW[u, k]  += sum_m g[m, u] h[m, k];  db[u] += sum_m g[m, u]  (the head's own gradients)
// A warp takes 32 consecutive rows at a time: lane l computes g of row l from
// coalesced loads of the per-row head values, then the warp walks the rows, four
// in flight, lane j owning columns CPL j .. CPL j + CPL - 1 (K = 32 CPL: one
// coalesced 256- or 512-byte row per access) and taking each row's g from its
// lane by shuffles.  Partial sums stay in registers until one shared-memory
// reduction over the block's 8 warps at the end.
template <int NO, int CPL>
__global__ void __launch_bounds__(256, CPL == 4 ? 3 : 2)
    head_bwd_fused_kernel(int64_t M, int K, const float* __restrict__ dsigma, const float* __restrict__ sraw,
                          const float* __restrict__ drgb, const float* __restrict__ rgb, const float* __restrict__ W,
                          const op16* __restrict__ h, op16* dz, float* colsum, float* dW, float* db, int fmt,
                          const float* gscale, int* found_inf) {
    constexpr int RPP = 4;   // rows in flight per warp
    __shared__ float red[8][256 + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const float gs0 = gscale ? gscale[0] : 1.f, gs1 = gscale ? gscale[1] : 1.f;
    const float vmax = tc::fmt_max(fmt);
    bool bad = false;
    float w[NO][CPL], dwl[NO][CPL], cs[CPL], dbl[NO];
#pragma unroll
    for (int u = 0; u < NO; ++u) {
        dbl[u] = 0.f;
#pragma unroll
        for (int i = 0; i < CPL; ++i) {
            w[u][i] = W[u * K + lane * CPL + i];
            dwl[u][i] = 0.f;
        }
    }
#pragma unroll
    for (int i = 0; i < CPL; ++i) cs[i] = 0.f;
    const int64_t gstride = int64_t(gridDim.x) * 8 * 32;
    for (int64_t base = (int64_t(blockIdx.x) * 8 + warp) * 32; base < M; base += gstride) {
        // g of row base + lane
        float gl[NO];
        {
            const int64_t r = base + lane;
#pragma unroll
            for (int u = 0; u < NO; ++u) gl[u] = 0.f;
            if (r < M) {
                int u0 = 0;
                if (NO == 4) {
                    gl[0] = sraw[r] > 0.f ? dsigma[r] : 0.f;
                    u0 = 1;
                }
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float v = rgb[3 * r + c];
                    gl[u0 + c] = drgb[3 * r + c] * v * (1.f - v);
                }
            }
#pragma unroll
            for (int u = 0; u < NO; ++u) dbl[u] += gl[u];
        }
        const int nrows = M - base < 32 ? int(M - base) : 32;
        for (int t0 = 0; t0 < nrows; t0 += RPP) {
            uint32_t raw[RPP][CPL / 2];
#pragma unroll
            for (int t = 0; t < RPP; ++t) {   // every row's loads before any row's arithmetic
                if (t0 + t >= nrows) continue;
                const op16* hr = h + (base + t0 + t) * K + lane * CPL;
                if (CPL == 8) {
                    const uint4 q = *reinterpret_cast<const uint4*>(hr);
                    raw[t][0] = q.x; raw[t][CPL / 2 > 1 ? 1 : 0] = q.y;
                    raw[t][CPL / 2 > 2 ? 2 : 0] = q.z; raw[t][CPL / 2 > 3 ? 3 : 0] = q.w;
                } else {
                    const uint2 q = *reinterpret_cast<const uint2*>(hr);
                    raw[t][0] = q.x; raw[t][CPL / 2 > 1 ? 1 : 0] = q.y;
                }
            }
#pragma unroll
            for (int t = 0; t < RPP; ++t) {
                float g[NO];   // row t0 + t's head gradients, from its lane
#pragma unroll
                for (int u = 0; u < NO; ++u) g[u] = __shfl_sync(0xffffffffu, gl[u], (t0 + t) & 31);
                if (t0 + t >= nrows) continue;
                uint32_t o[CPL / 2];
#pragma unroll
                for (int p = 0; p < CPL / 2; ++p) {
                    const float2 hx = tc::unpack16(raw[t][p], fmt);
                    float v0 = 0.f, v1 = 0.f;
#pragma unroll
                    for (int u = 0; u < NO; ++u) {
                        v0 += g[u] * w[u][2 * p];
                        v1 += g[u] * w[u][2 * p + 1];
                        dwl[u][2 * p] += g[u] * hx.x;
                        dwl[u][2 * p + 1] += g[u] * hx.y;
                    }
                    v0 = hx.x > 0.f ? v0 * gs0 : 0.f;
                    v1 = hx.y > 0.f ? v1 * gs0 : 0.f;
                    cs[2 * p] += v0;
                    cs[2 * p + 1] += v1;
                    bad |= !(fabsf(v0) <= vmax) || !(fabsf(v1) <= vmax);
                    o[p] = tc::pack16(v0, v1, fmt);
                }
                op16* dr = dz + (base + t0 + t) * K + lane * CPL;
                if (CPL == 8) *reinterpret_cast<uint4*>(dr) = make_uint4(o[0], o[CPL / 2 > 1 ? 1 : 0],
                                                                         o[CPL / 2 > 2 ? 2 : 0], o[CPL / 2 > 3 ? 3 : 0]);
                else *reinterpret_cast<uint2*>(dr) = make_uint2(o[0], o[CPL / 2 > 1 ? 1 : 0]);
            }
        }
    }
    // block sums over the 8 warps, one K-vector at a time, then one atomic per column
    auto reduce = [&](const float (&vals)[CPL], float* dst, float scale) {
#pragma unroll
        for (int i = 0; i < CPL; ++i) red[warp][lane * CPL + i] = vals[i];
        __syncthreads();
        for (int k = threadIdx.x; k < K; k += blockDim.x) {
            float sum = 0.f;
#pragma unroll
            for (int ww = 0; ww < 8; ++ww) sum += red[ww][k];
            atomicAdd(dst + k, sum * scale);
        }
        __syncthreads();
    };
    if (found_inf && bad) atomicExch(found_inf, 1);
    if (colsum) reduce(cs, colsum, gs1);
#pragma unroll
    for (int u = 0; u < NO; ++u) reduce(dwl[u], dW + u * K, 1.f);
#pragma unroll
    for (int u = 0; u < NO; ++u) {
        float v = dbl[u];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) atomicAdd(db + u, v);
    }
}

template <int NO>
int head_bwd_fused(int64_t M, int K, const float* dsigma, const float* sraw, const float* drgb, const float* rgb,
                   const float* W, const op16* h, op16* dz, float* colsum, float* dW, float* db, int fmt,
                   const float* gscale, int* found_inf, cudaStream_t s) {
    if (K != 128 && K != 256) return SRF_ERR_UNSUPPORTED;
    if (M <= 0) return SRF_OK;
    int64_t blocks = (M + 255) / 256;   // 8 warps of 32 rows
    if (blocks > int64_t(num_sms()) * 8) blocks = int64_t(num_sms()) * 8;
    if (K == 128)
        head_bwd_fused_kernel<NO, 4><<<unsigned(blocks), 256, 0, s>>>(M, K, dsigma, sraw, drgb, rgb, W, h, dz, colsum,
                                                                     dW, db, fmt, gscale, found_inf);
    else
        head_bwd_fused_kernel<NO, 8><<<unsigned(blocks), 256, 0, s>>>(M, K, dsigma, sraw, drgb, rgb, W, h, dz, colsum,
                                                                     dW, db, fmt, gscale, found_inf);
    return launch_status();
}

// Sigma head gradients (SimpleNeRF17.py:735-741 adjoint): with g[m] = dsigma[m] when
// the raw sigma is positive (the ReLU), else 0, dW[k] += sum_m g[m] h[m, k] and
// db += sum_m g[m] over the last trunk layer's stored 16-bit rows h (K columns,
// K = 8 x 32).  A warp takes 32 consecutive rows: lane l computes g of row l from
// coalesced loads, then the warp walks the rows, four in flight, 8 columns a lane,
// taking each row's g by a shuffle; the block's sums go out with one atomic per column.
__global__ void __launch_bounds__(256) sigma_head_wgrad_kernel(int64_t M, int K, const float* __restrict__ dsigma,
                                                               const float* __restrict__ sraw,
                                                               const op16* __restrict__ h, float* dW, float* db,
                                                               int fmt) {
    constexpr int RPP = 4;
    __shared__ float red[8][256 + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, gsum = 0.f;
    const int64_t gstride = int64_t(gridDim.x) * 8 * 32;
    for (int64_t base = (int64_t(blockIdx.x) * 8 + warp) * 32; base < M; base += gstride) {
        const int64_t rl = base + lane;
        const float gl = rl < M && sraw[rl] > 0.f ? dsigma[rl] : 0.f;
        gsum += gl;
        const int nrows = M - base < 32 ? int(M - base) : 32;
        for (int t0 = 0; t0 < nrows; t0 += RPP) {
            uint4 raw[RPP];
#pragma unroll
            for (int t = 0; t < RPP; ++t)
                if (t0 + t < nrows) raw[t] = *reinterpret_cast<const uint4*>(h + (base + t0 + t) * K + lane * 8);
#pragma unroll
            for (int t = 0; t < RPP; ++t) {
                const float g = __shfl_sync(0xffffffffu, gl, (t0 + t) & 31);
                if (t0 + t >= nrows || g == 0.f) continue;
                const uint32_t w4[4] = {raw[t].x, raw[t].y, raw[t].z, raw[t].w};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const float2 f = tc::unpack16(w4[q], fmt);
                    acc[2 * q] += g * f.x;
                    acc[2 * q + 1] += g * f.y;
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) red[warp][lane * 8 + i] = acc[i];
    __syncthreads();
    if (threadIdx.x < K) {
        float s = 0.f;
#pragma unroll
        for (int w = 0; w < 8; ++w) s += red[w][threadIdx.x];
        atomicAdd(dW + threadIdx.x, s);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gsum += __shfl_xor_sync(0xffffffffu, gsum, o);
    if (lane == 0) atomicAdd(db, gsum);
}

int sigma_head_wgrad(int64_t M, int K, const float* dsigma, const float* sraw, const op16* h, float* dW, float* db,
                     int fmt, cudaStream_t s) {
    if (K != 256) return SRF_ERR_UNSUPPORTED;
    if (M <= 0) return SRF_OK;
    int64_t blocks = (M + 255) / 256;   // 8 warps of 32 rows
    if (blocks > int64_t(num_sms()) * 6) blocks = int64_t(num_sms()) * 6;
    sigma_head_wgrad_kernel<<<unsigned(blocks), 256, 0, s>>>(M, K, dsigma, sraw, h, dW, db, fmt);
    return launch_status();
}

int pad64(int x) { return (x + 63) / 64 * 64; }

// ------------------------------------------------------------ layout -------

struct TcLayout {
    int enc_w, vx_w;
    std::vector<LayerMap> trunk, view;
    LayerMap feat;
    bool ok;
    explicit TcLayout(const MlpLayout& L) {
        enc_w = pad64(L.ppe);
        vx_w = L.vdep ? pad64(L.vin > 0 ? L.vin : 1) : 0;
        ok = (L.Wp == 64 || L.Wp == 128 || L.Wp == 256) && (!L.vdep || L.Wv == 64 || L.Wv == 128 || L.Wv == 256);
        for (int j = 0; j < L.Dp; ++j) {
            LayerMap m{};
            m.n = L.Wp;
            if (j == 0) {
                m.nsrc = 1;
                m.pad0[0] = 0; m.padw[0] = enc_w; m.ref0[0] = 0; m.refw[0] = L.pin;
            } else if (j - 1 == L.skip) {
                m.nsrc = 2;
                m.pad0[0] = 0; m.padw[0] = enc_w; m.ref0[0] = 0; m.refw[0] = L.pin;
                m.pad0[1] = enc_w; m.padw[1] = L.Wp; m.ref0[1] = L.pin; m.refw[1] = L.Wp;
            } else {
                m.nsrc = 1;
                m.pad0[0] = 0; m.padw[0] = L.Wp; m.ref0[0] = 0; m.refw[0] = L.Wp;
            }
            trunk.push_back(m);
        }
        feat = LayerMap{};
        feat.n = L.Wp; feat.nsrc = 1; feat.padw[0] = L.Wp; feat.refw[0] = L.Wp;
        if (L.vdep) {
            for (int j = 0; j < L.Dv; ++j) {
                LayerMap m{};
                m.n = L.Wv;
                if (j == 0) {
                    m.nsrc = L.vin > 0 ? 2 : 1;
                    m.pad0[0] = 0; m.padw[0] = L.Wp; m.ref0[0] = 0; m.refw[0] = L.Wp;
                    if (L.vin > 0) { m.pad0[1] = L.Wp; m.padw[1] = vx_w; m.ref0[1] = L.Wp; m.refw[1] = L.vin; }
                } else {
                    m.nsrc = 1;
                    m.pad0[0] = 0; m.padw[0] = L.Wv; m.ref0[0] = 0; m.refw[0] = L.Wv;
                }
                view.push_back(m);
            }
        }
        for (auto& m : trunk) ok = ok && m.kpad() <= 512;
        for (auto& m : view) ok = ok && m.kpad() <= 512;
    }
};

struct TcWs {
    op16* enc; op16* vext;
    std::vector<op16*> h, hv;
    std::vector<uint32_t*> hbits;   // ReLU bits of h[j] for the backward-data masks (backward only)
    op16* feat;
    float* sraw; float* rgb;
    std::vector<op16*> W, WT, Wv, WTv;
    op16* Wf; op16* WTf;
    op16* dz0; op16* dz1; op16* dfeat;
    float* dsig; float* dout; float* partial; size_t partial_floats;
};

size_t carve_tc(const MlpLayout& L, const TcLayout& T, int64_t m, bool bwd, void* base, size_t cap, TcWs* out) {
    Carver c(base, cap);
    TcWs w;
    w.enc = c.take<op16>(size_t(m) * T.enc_w);
    w.vext = L.vdep ? c.take<op16>(size_t(m) * T.vx_w) : nullptr;
    if (bwd) {
        // the backward reads every layer's activation
        for (int j = 0; j < L.Dp; ++j) w.h.push_back(c.take<op16>(size_t(m) * L.Wp));
        w.feat = L.vdep ? c.take<op16>(size_t(m) * L.Wp) : nullptr;
        for (int j = 0; L.vdep && j < L.Dv; ++j) w.hv.push_back(c.take<op16>(size_t(m) * L.Wv));
    } else {
        // forward only: layer j reads only layer j-1 (the skip input is the
        // encoding, kept separately), so two activation buffers alternate
        op16* ping = c.take<op16>(size_t(m) * L.Wp);
        op16* pong = L.Dp > 1 || L.vdep ? c.take<op16>(size_t(m) * L.Wp) : ping;
        for (int j = 0; j < L.Dp; ++j) w.h.push_back(j & 1 ? pong : ping);
        // feature layer reads h[Dp-1]; the view layers read the feature, then each other
        op16* other = (L.Dp - 1) & 1 ? ping : pong;
        w.feat = L.vdep ? other : nullptr;
        op16* hv0 = (L.vdep && L.Dv > 0) ? c.take<op16>(size_t(m) * L.Wv) : nullptr;
        op16* hv1 = (L.vdep && L.Dv > 1) ? c.take<op16>(size_t(m) * L.Wv) : hv0;
        for (int j = 0; L.vdep && j < L.Dv; ++j) w.hv.push_back(j & 1 ? hv1 : hv0);
    }
    w.sraw = c.take<float>(size_t(m));
    w.rgb = c.take<float>(size_t(m) * 3);
    for (auto& lm : T.trunk) {
        w.W.push_back(c.take<op16>(size_t(lm.n) * lm.kpad()));
        w.WT.push_back(c.take<op16>(size_t(lm.n) * lm.kpad()));
    }
    w.Wf = c.take<op16>(size_t(L.Wp) * L.Wp);
    w.WTf = c.take<op16>(size_t(L.Wp) * L.Wp);
    for (auto& lm : T.view) {
        w.Wv.push_back(c.take<op16>(size_t(lm.n) * lm.kpad()));
        w.WTv.push_back(c.take<op16>(size_t(lm.n) * lm.kpad()));
    }
    int wmax = L.Wp > L.Wv ? L.Wp : L.Wv;
    if (bwd) {
        // h[j] feeds trunk layer j + 1's mask, and h[Dp - 1] the feature layer's (view-dependent nets)
        for (int j = 0; j < L.Dp; ++j) w.hbits.push_back(c.take<uint32_t>(size_t(m) * (L.Wp / 32)));
        w.dz0 = c.take<op16>(size_t(m) * wmax);
        w.dz1 = c.take<op16>(size_t(m) * wmax);
        w.dfeat = L.vdep ? c.take<op16>(size_t(m) * L.Wp) : nullptr;
        w.dsig = c.take<float>(size_t(m));
        w.dout = c.take<float>(size_t(m) * 4);
        w.partial_floats = tc_wgrad_partial_floats(wmax, 512);
        w.partial = c.take<float>(w.partial_floats);
    } else {
        w.dz0 = w.dz1 = w.dfeat = nullptr;
        w.dsig = w.dout = w.partial = nullptr;
        w.partial_floats = 0;
    }
    if (out) *out = w;
    return c.used;
}

int pack(const LayerMap& lm, const float* w, op16* wp, op16* wt, int fmt, cudaStream_t s) {
    dim3 grid((lm.kpad() + 127) / 128, lm.n);
    pack_weight_kernel<<<grid, 128, 0, s>>>(lm, w, wp, wt, fmt);
    return launch_status();
}

// Every layer of an MLP packed in ceil(layers / kPackBatch) launches.
int pack_all(const std::vector<LayerMap>& lms, const std::vector<const float*>& ws, const std::vector<op16*>& wps,
             const std::vector<op16*>& wts, int fmt, cudaStream_t s) {
    for (size_t i0 = 0; i0 < lms.size(); i0 += kPackBatch) {
        PackBatch b{};
        int kmax = 0, nmax = 0, cnt = 0;
        for (size_t i = i0; i < lms.size() && cnt < kPackBatch; ++i, ++cnt) {
            b.lm[cnt] = lms[i];
            b.w[cnt] = ws[i];
            b.wp[cnt] = wps[i];
            b.wt[cnt] = wts[i];
            kmax = lms[i].kpad() > kmax ? lms[i].kpad() : kmax;
            nmax = lms[i].n > nmax ? lms[i].n : nmax;
        }
        dim3 grid((kmax + 127) / 128, nmax, cnt);
        pack_weights_kernel<<<grid, 128, 0, s>>>(b, fmt);
        int st = launch_status();
        if (st) return st;
    }
    return SRF_OK;
}

// Operand format and loss scaler of one forward/backward call.
struct TcCtx {
    int fmt;
    srf_loss_scaler* scaler;   // {scale, 1/scale, found_inf, growth}; required by the FP16 backward
    const float* gscale() const { return scaler ? &scaler->scale : nullptr; }
    int* found_inf() const { return scaler ? &scaler->found_inf : nullptr; }
};

// The layer's weight gradient and, when bias_grad is given, its bias gradient (the
// sum of dZ over the samples, from the same tensor-core pass).
int wgrad_layer(const LayerMap& lm, float* partial, size_t partial_floats, const op16* dz, const op16* x0,
                int64_t ld0, const op16* x1, int64_t ld1, int64_t M, float* grad, const TcCtx& cx, cudaStream_t s,
                float* bias_grad = nullptr) {
    int splits = 0;
    int st = tc_wgrad(partial, partial_floats, dz, lm.n, lm.n, x0, ld0, lm.padw[0], x1, ld1,
                      lm.nsrc > 1 ? lm.padw[1] : 0, M, &splits, s, cx.fmt, bias_grad, cx.gscale());
    if (st) return st;
    dim3 grid((lm.kpad() + 127) / 128, lm.n);
    reduce_wgrad_kernel<<<grid, 128, 0, s>>>(lm, partial, splits, lm.n, grad, cx.gscale());
    return launch_status();
}

// Which forwards run as the one fused kernel (tc::mlp_fused_kernel) where the
// layout fits it: 0 none (one kernel per layer), 1 forward-only calls (default),
// 2 also the forward of a training step (which stores the activations the
// backward reads; slower than the per-layer kernels: its row-wise stores from the
// epilogue registers cost more than the reads they save).
std::atomic<int> g_mlp_fused{1};

// The fused kernel's layouts: 256-wide trunk of at most 8 layers, a point
// encoding of at most 64 columns feeding the first layer (and the skip layer)
// whole, and either no view branch (sigma + rgb on the last trunk layer) or the
// reference's single 128-wide view layer on [feature, PE(view dirs)] with at most
// 64 encoding columns.
bool fused_fits(const MlpLayout& L, const TcLayout& T) {
    if (L.Wp != 256 || T.enc_w != 64 || L.pin != L.ppe || L.Dp < 1 || L.desc.points_pe_degree > 10) return false;
    if (L.skip >= 0 && L.skip >= L.Dp - 1) return false;
    if (L.vdep && (L.Dv != 1 || L.Wv != 128 || T.vx_w != 64 || L.vin != L.vpe || L.vpe <= 0 ||
                   L.desc.views_pe_degree > 10))
        return false;
    return L.Dp + (L.vdep ? 2 : 0) <= tc::kFusedMaxLayers;
}

// The whole forward in one launch: the layer program of the kernel from the
// per-layer description, the weight maps, and with store the maps of every
// activation the backward reads (same buffers and layouts as the per-layer path).
int launch_fused(const MlpLayout& L, const TcLayout& T, const float* const* P, const TcWs& w, int64_t m,
                 const float* noise, float* sigma, float* rgb, bool store, const TcCtx& cx, cudaStream_t s) {
    if (m <= 0) return SRF_OK;
    tc::FusedProgram pr{};
    static tc::FusedMaps maps_zero{};
    tc::FusedMaps maps = maps_zero;
    int head_off = 0, bias_off = 0;
    const int last_enc = L.skip >= 0 ? L.skip + 1 : 0;   // the last layer that reads PE(points)
    auto add = [&](int kind, const op16* wp, int kpad, int n, int ext_kb, int ext_src, int ext_wait, int head,
                   const float* bias, const float* hw, const float* hb, int enc_last, op16* out, uint32_t* bits) {
        const int l = pr.nl++;
        tc::FusedLayer& F = pr.layer[l];
        F.kind = kind;
        F.kb = kpad / 64;
        F.ext_kb = ext_kb;
        F.ext_src = ext_src;
        F.ext_wait = ext_wait;
        F.n = n;
        F.head = head;
        F.enc_last = enc_last;
        F.bias_off = bias_off;
        F.head_off = head_off;
        bias_off += n;
        head_off += tc::head_units(head) * n;
        pr.bias[l] = bias;
        pr.head_w[l] = hw;
        pr.head_b[l] = hb;
        pr.bits_out[l] = store ? bits : nullptr;
        pr.out[l] = store ? out : nullptr;
        return make_map(&maps.w[l], wp, uint64_t(kpad), uint64_t(n), uint64_t(kpad) * 2, 64, uint32_t(n));
    };
    bool ok = true;
    for (int j = 0; j < L.Dp; ++j) {
        const bool last = j == L.Dp - 1;
        const int head = last ? (L.vdep ? tc::kHeadSigma : tc::kHeadSigmaRgb) : tc::kHeadNone;
        const int kind = last ? (L.vdep ? tc::kFusedSigma : tc::kFusedSigmaRgb) : tc::kFusedPlain;
        const bool enc_in = j == 0 || j - 1 == L.skip;
        ok = ok && add(kind, w.W[j], T.trunk[j].kpad(), 256, enc_in ? 0 : -1, 0, j == 0, head, P[L.idx_trunk_w(j) + 1],
                       last ? P[L.idx_out_w()] : nullptr, last ? P[L.idx_out_w() + 1] : nullptr, j == last_enc,
                       w.h[j], (j + 1 < L.Dp || L.vdep) && store ? w.hbits[j] : nullptr);
    }
    if (L.vdep) {
        ok = ok && add(tc::kFusedLinear, w.Wf, L.Wp, 256, -1, 0, 0, tc::kHeadNone, P[L.idx_feat_w() + 1], nullptr,
                       nullptr, 0, w.feat, nullptr);
        ok = ok && add(tc::kFusedView, w.Wv[0], T.view[0].kpad(), 128, 4, 1, 1, tc::kHeadRgb, P[L.idx_view_w(0) + 1],
                       P[L.idx_rgb_w()], P[L.idx_rgb_w() + 1], 0, w.hv[0], nullptr);
    }
    if (!ok) return SRF_ERR_CUDA;
    if (head_off > tc::kFusedHeadFloats || bias_off > tc::kFusedBiasFloats) return SRF_ERR_UNSUPPORTED;
    // the encodings the standalone encoder wrote: [m, 64] 16-bit rows, 128-row boxes
    if (!make_map(&maps.enc, w.enc, uint64_t(T.enc_w), uint64_t(m), uint64_t(T.enc_w) * 2, 64, 128))
        return SRF_ERR_CUDA;
    if (L.vdep && !make_map(&maps.vx, w.vext, uint64_t(T.vx_w), uint64_t(m), uint64_t(T.vx_w) * 2, 64, 128))
        return SRF_ERR_CUDA;
    pr.fmt = cx.fmt;
    pr.has_vx = L.vdep ? 1 : 0;
    // the next tile's ENC once the tile's last ENC reader is two layers back (its MMAs are
    // then complete), VX two layers into the tile (the previous tile's view layer is done)
    pr.enc_at = last_enc + 2 < pr.nl ? last_enc + 2 : pr.nl;
    pr.vx_at = pr.nl - 1 < 2 ? pr.nl - 1 : 2;
    pr.has_noise = noise != nullptr;
    pr.M = m;
    pr.noise = noise;
    pr.sraw = w.sraw;
    pr.sigma = sigma;
    pr.rgb_ws = w.rgb;
    pr.rgb_out = rgb;
    pr.found_inf = cx.found_inf();
    pr.flag = device_flag();
    static bool attr_done[2] = {false, false};
    auto kern = store ? tc::mlp_fused_kernel<true> : tc::mlp_fused_kernel<false>;
    if (!attr_done[store]) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tc::kFusedSmem));
        if (e != cudaSuccess) {
            set_cuda_error(e);
            return SRF_ERR_CUDA;
        }
        attr_done[store] = true;
    }
    const int64_t tiles = (m + 127) / 128;
    const int grid = int(tiles < num_sms() ? tiles : num_sms());
    kern<<<grid, tc::kFusedThreads, tc::kFusedSmem, s>>>(maps, pr);
    return launch_status();
}

}  // namespace

size_t mlp_tc_workspace(const MlpLayout& L, int64_t m, bool bwd) {
    TcLayout T(L);
    if (!T.ok) return 0;
    return carve_tc(L, T, m, bwd, nullptr, ~size_t(0), nullptr);
}

int mlp_tc_forward(const MlpLayout& L, const float* const* P, const float* pts, const float* dirs, int dir_div,
                   int64_t m, const float* noise, float* sigma, float* rgb, bool bwd, void* ws, size_t ws_bytes,
                   int fmt, srf_loss_scaler* scaler, cudaStream_t s) {
    const TcCtx cx{fmt, scaler};
    TcLayout T(L);
    if (!T.ok) return SRF_ERR_UNSUPPORTED;
    TcWs w;
    if (carve_tc(L, T, m, bwd, ws, ws_bytes, &w) > ws_bytes) return SRF_ERR_WORKSPACE;
    int st;
    {
        std::vector<LayerMap> lms;
        std::vector<const float*> ws;
        std::vector<op16*> wps, wts;
        for (int j = 0; j < L.Dp; ++j) {
            lms.push_back(T.trunk[j]);
            ws.push_back(P[L.idx_trunk_w(j)]);
            wps.push_back(w.W[j]);
            wts.push_back(w.WT[j]);
        }
        if (L.vdep) {
            lms.push_back(T.feat);
            ws.push_back(P[L.idx_feat_w()]);
            wps.push_back(w.Wf);
            wts.push_back(w.WTf);
            for (int j = 0; j < L.Dv; ++j) {
                lms.push_back(T.view[j]);
                ws.push_back(P[L.idx_view_w(j)]);
                wps.push_back(w.Wv[j]);
                wts.push_back(w.WTv[j]);
            }
        }
        if ((st = pack_all(lms, ws, wps, wts, fmt, s))) return st;
    }
    {
        const int vx = L.vdep ? T.vx_w : 0;
        const size_t smem = size_t(kEncRows) * (T.enc_w + vx + 2) * sizeof(op16);
        encode16_kernel<<<unsigned((m + kEncRows - 1) / kEncRows), kEncRows, smem, s>>>(
            pts, L.vpe ? dirs : nullptr, dir_div, m, L.desc.points_pe_degree, L.desc.views_pe_degree, L.pin, T.enc_w,
            vx, w.enc, L.vdep ? w.vext : nullptr, fmt);
    }
    if ((st = launch_status())) return st;
    const int fused = g_mlp_fused.load();
    if (fused >= (bwd ? 2 : 1) && fused_fits(L, T)) return launch_fused(L, T, P, w, m, noise, sigma, rgb, bwd, cx, s);
    for (int j = 0; j < L.Dp; ++j) {
        const LayerMap& lm = T.trunk[j];
        const op16* x0 = j == 0 || j - 1 == L.skip ? w.enc : w.h[j - 1];
        int64_t ld0 = j == 0 || j - 1 == L.skip ? T.enc_w : L.Wp;
        const op16* x1 = lm.nsrc > 1 ? w.h[j - 1] : nullptr;
        tc::GemmEpilogue ep = make_epilogue(w.h[j], L.Wp, P[L.idx_trunk_w(j) + 1], 1, fmt, cx.found_inf());
        if (bwd && (j + 1 < L.Dp || L.vdep)) {   // the backward-data pass after h[j] masks with these bits
            ep.bits_out = w.hbits[j];
            ep.ld_bits = L.Wp / 32;
        }
        if (j == L.Dp - 1) {
            // sigma head (and, without view dependence, the rgb head) on the last trunk layer's rows
            ep.head_mode = L.vdep ? tc::kHeadSigma : tc::kHeadSigmaRgb;
            ep.head_w = P[L.idx_out_w()];
            ep.head_b = P[L.idx_out_w() + 1];
            ep.head_noise = noise;
            ep.head_sraw = w.sraw;
            ep.head_sigma = sigma;
            ep.head_rgb_ws = w.rgb;
            ep.head_rgb_out = rgb;
        }
        st = tc_linear(ep, x0, ld0, lm.padw[0], x1, L.Wp, lm.nsrc > 1 ? lm.padw[1] : 0, w.W[j], lm.kpad(), lm.n, 0, m,
                       lm.n, s);
        if (st) return st;
    }
    if (!L.vdep) return SRF_OK;
    const op16* hl = w.h[L.Dp - 1];
    st = tc_linear(make_epilogue(w.feat, L.Wp, P[L.idx_feat_w() + 1], 0, fmt, cx.found_inf()), hl, L.Wp, L.Wp,
                   nullptr, 0, 0, w.Wf, L.Wp, L.Wp, 0, m, L.Wp, s);
    if (st) return st;
    for (int j = 0; j < L.Dv; ++j) {
        const LayerMap& lm = T.view[j];
        const op16* x0 = j == 0 ? w.feat : w.hv[j - 1];
        int64_t ld0 = j == 0 ? L.Wp : L.Wv;
        tc::GemmEpilogue ep = make_epilogue(w.hv[j], L.Wv, P[L.idx_view_w(j) + 1], 1, fmt, cx.found_inf());
        if (j == L.Dv - 1) {
            ep.head_mode = tc::kHeadRgb;
            ep.head_w = P[L.idx_rgb_w()];
            ep.head_b = P[L.idx_rgb_w() + 1];
            ep.head_rgb_ws = w.rgb;
            ep.head_rgb_out = rgb;
        }
        st = tc_linear(ep, x0, ld0, lm.padw[0], lm.nsrc > 1 ? w.vext : nullptr, T.vx_w, lm.nsrc > 1 ? lm.padw[1] : 0,
                       w.Wv[j], lm.kpad(), lm.n, 0, m, lm.n, s);
        if (st) return st;
    }
    return SRF_OK;
}

int mlp_tc_backward(const MlpLayout& L, const float* const* P, const float* dsigma, const float* drgb, int64_t m,
                    int dir_div, float* const* G, void* ws, size_t ws_bytes, int fmt, srf_loss_scaler* scaler,
                    cudaStream_t s) {
    (void)dir_div;
    const TcCtx cx{fmt, scaler};
    // a dgrad epilogue in this call's format, with the loss scale applied
    auto bwd_epilogue = [&](op16* out, int64_t ld) {
        tc::GemmEpilogue ep = make_epilogue(out, ld, nullptr, 0, fmt, cx.found_inf());
        ep.gscale = cx.gscale();
        return ep;
    };
    TcLayout T(L);
    if (!T.ok) return SRF_ERR_UNSUPPORTED;
    TcWs w;
    if (carve_tc(L, T, m, true, ws, ws_bytes, &w) > ws_bytes) return SRF_ERR_WORKSPACE;
    int st;
    op16* dz = w.dz0;
    op16* dz2 = w.dz1;
    const op16* hl = w.h[L.Dp - 1];
    if (L.vdep) {
        // rgb head: dZ of the last view layer, its bias gradient, the head's dW/db
        st = head_bwd_fused<3>(m, L.Wv, nullptr, nullptr, drgb, w.rgb, P[L.idx_rgb_w()], w.hv[L.Dv - 1], dz,
                               nullptr, G[L.idx_rgb_w()], G[L.idx_rgb_w() + 1], fmt, cx.gscale(), cx.found_inf(),
                               s);
        if (st) return st;
        for (int j = L.Dv - 1; j >= 0; --j) {
            const LayerMap& lm = T.view[j];
            const op16* x0 = j == 0 ? w.feat : w.hv[j - 1];
            int64_t ld0 = j == 0 ? L.Wp : L.Wv;
            st = wgrad_layer(lm, w.partial, w.partial_floats, dz, x0, ld0, lm.nsrc > 1 ? w.vext : nullptr, T.vx_w,
                             m, G[L.idx_view_w(j)], cx, s, G[L.idx_view_w(j) + 1]);
            if (st) return st;
            if (j > 0) {
                tc::GemmEpilogue ep = bwd_epilogue(dz2, L.Wv);
                ep.mask = w.hv[j - 1];
                ep.ld_mask = L.Wv;
                st = tc_linear(ep, dz, L.Wv, L.Wv, nullptr, 0, 0, w.WTv[j], L.Wv, lm.kpad(), 0, m, L.Wv, s);
                if (st) return st;
                std::swap(dz, dz2);
            } else {
                tc::GemmEpilogue ep = bwd_epilogue(w.dfeat, L.Wp);
                st = tc_linear(ep, dz, L.Wv, L.Wv, nullptr, 0, 0, w.WTv[0], L.Wv, lm.kpad(), 0, m, L.Wp, s);
                if (st) return st;
            }
        }
        st = wgrad_layer(T.feat, w.partial, w.partial_floats, w.dfeat, hl, L.Wp, nullptr, 0, m, G[L.idx_feat_w()],
                         cx, s, G[L.idx_feat_w() + 1]);
        if (st) return st;
        // feature-layer dgrad with the sigma head's adjoint fused in: dZ_last =
        // (dfeat . Wf + dsig w_sigma) * (h_last > 0), dsig = dsigma * (sraw > 0);
        // the same pass adds the sigma head's weight (sum dsig h_last) and bias gradients
        tc::GemmEpilogue ep = bwd_epilogue(dz, L.Wp);
        ep.mask_bits = w.hbits[L.Dp - 1];
        ep.ld_bits = L.Wp / 32;
        ep.r1_row = dsigma;
        ep.r1_gate = w.sraw;
        ep.r1_col = P[L.idx_out_w()];
        st = tc_linear(ep, w.dfeat, L.Wp, L.Wp, nullptr, 0, 0, w.WTf, L.Wp, L.Wp, 0, m, L.Wp, s);
        if (st) return st;
        st = sigma_head_wgrad(m, L.Wp, dsigma, w.sraw, hl, G[L.idx_out_w()], G[L.idx_out_w() + 1], fmt, s);
        if (st) return st;
    } else {
        st = head_bwd_fused<4>(m, L.Wp, dsigma, w.sraw, drgb, w.rgb, P[L.idx_out_w()], hl, dz, nullptr,
                               G[L.idx_out_w()], G[L.idx_out_w() + 1], fmt, cx.gscale(), cx.found_inf(), s);
        if (st) return st;
    }
    for (int j = L.Dp - 1; j >= 0; --j) {
        const LayerMap& lm = T.trunk[j];
        const op16* x0 = j == 0 || j - 1 == L.skip ? w.enc : w.h[j - 1];
        int64_t ld0 = j == 0 || j - 1 == L.skip ? T.enc_w : L.Wp;
        st = wgrad_layer(lm, w.partial, w.partial_floats, dz, x0, ld0, lm.nsrc > 1 ? w.h[j - 1] : nullptr, L.Wp, m,
                         G[L.idx_trunk_w(j)], cx, s, G[L.idx_trunk_w(j) + 1]);
        if (st) return st;
        if (j == 0) break;
        int row0 = lm.nsrc > 1 ? lm.padw[0] : 0;
        tc::GemmEpilogue ep = bwd_epilogue(dz2, L.Wp);
        ep.mask_bits = w.hbits[j - 1];
        ep.ld_bits = L.Wp / 32;
        st = tc_linear(ep, dz, L.Wp, L.Wp, nullptr, 0, 0, w.WT[j], L.Wp, lm.kpad(), row0, m, L.Wp, s);
        if (st) return st;
        std::swap(dz, dz2);
    }
    return SRF_OK;
}

// ======================================================================
// TensoRF renderer on tcgen05: basis_matrix_color (C -> F, no bias) and
// MlpFeaturesColorPredictor (SimpleTensoRF09.py:1151, 1370-1421):
//   B = feats . Wb^T;  x = [PE(B, Lf), PE(view, Lv)];  h1 = relu(x W1^T + b1);
//   h2 = relu(h1 W2^T + b2);  rgb = sigmoid(h2 W3^T + b3)
// The basis and the encodings run in one SIMT pass (3,888 MAC per sample for
// C = 144, F = 27) that writes x as a 16-bit row padded to a multiple of 64;
// the two U-wide layers are tcgen05 GEMMs with the rgb head fused into the
// second one's epilogue.  The backward mirrors the NeRF path, then the PE
// adjoint and the basis layer's FP32 backward give d feats for the VM adjoint.
// ======================================================================

namespace {

constexpr int kMaxBasis = 32;    // largest basis width (features_dimension_color) it holds in registers

// The renderer's 16-bit input rows x (k1p columns): the 2 lf + 1 feature blocks
// [B, sin B, cos B, sin 2B, cos 2B, ...] (the reference's PE order) each at a
// column stride bw = F rounded up to 8 (so every block starts on a 16-byte
// boundary and can be written as whole vectors), the view block [d, sin d, cos d,
// ...] from column v0, zeros up to k1p; the packed W1 holds zero columns in the
// gaps.  B rows (the basis outputs kept for the PE adjoint) have kMaxBasis floats.
struct RenderLayout {
    int C, F, U, lf, lv, view, k1, k1p, bw, bs, v0;
    LayerMap l1, l2;
    bool ok;
    RenderLayout(int c, int f, int u, int lf_, int lv_, int view_) : C(c), F(f), U(u), lf(lf_), lv(lv_), view(view_) {
        k1 = F * (2 * lf + 1) + (view ? 3 * (2 * lv + 1) : 0);
        bw = (F + 7) / 8 * 8;
        bs = kMaxBasis;
        v0 = bw * (2 * lf + 1);
        k1p = pad64(v0 + (view ? 3 * (2 * lv + 1) : 0));
        l1 = LayerMap{};
        l1.n = U; l1.nsrc = 1; l1.padw[0] = k1p; l1.refw[0] = k1;
        l1.nblk = 2 * lf + 1; l1.bwp = bw; l1.bwr = F;
        l2 = LayerMap{};
        l2.n = U; l2.nsrc = 1; l2.padw[0] = U; l2.refw[0] = U;
        ok = (U == 128 || U == 256) && C >= 4 && C <= 1024 && C % 4 == 0 && F >= 1 && F <= kMaxBasis && k1p <= 256 &&
             lf >= 0 &&
             lv >= 0 && lf <= 10 && lv <= 10;
    }
};

struct RenderWs {
    float* B;        // (m, bs) basis outputs (kept for the PE adjoint)
    op16* x;         // (m, k1p)
    op16* h1;        // (m, U)
    op16* h2;        // (m, U)
    float* rgb;      // (m, 3)
    op16 *W1, *W1T, *W2, *W2T;
    float* WbT;      // (C, kMaxBasis)
    op16 *dz0, *dz1, *dx;   // (m, U), (m, U), (m, k1p)
    float* dB;              // (m, kMaxBasis) basis-output gradients of the tensor-core adjoint
    float* partial;
    size_t partial_floats;
};

size_t carve_render(const RenderLayout& R, int64_t m, bool bwd, void* base, size_t cap, RenderWs* out) {
    Carver c(base, cap);
    RenderWs w{};
    w.B = c.take<float>(size_t(m) * R.bs);
    w.x = c.take<op16>(size_t(m) * R.k1p);
    w.h1 = c.take<op16>(size_t(m) * R.U);
    w.h2 = c.take<op16>(size_t(m) * R.U);
    w.rgb = c.take<float>(size_t(m) * 3);
    w.W1 = c.take<op16>(size_t(R.U) * R.k1p);
    w.W1T = c.take<op16>(size_t(R.U) * R.k1p);
    w.W2 = c.take<op16>(size_t(R.U) * R.U);
    w.W2T = c.take<op16>(size_t(R.U) * R.U);
    w.WbT = c.take<float>(size_t(R.C) * kMaxBasis);
    if (bwd) {
        w.dz0 = c.take<op16>(size_t(m) * R.U);
        w.dz1 = c.take<op16>(size_t(m) * R.U);
        w.dx = c.take<op16>(size_t(m) * R.k1p);
        w.dB = c.take<float>(size_t(m) * kMaxBasis);
        w.partial_floats = tc_wgrad_partial_floats(R.U, 256);
        w.partial = c.take<float>(w.partial_floats);
    }
    if (out) *out = w;
    return c.used;
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// B = feats . Wb^T (FP32) and x = [PE(B, lf), PE(view, lv), 0...] in format fmt,
// a persistent pass over tiles of NT / 8 * RPT samples (NT threads; 128 threads x 2
// rows, four blocks per SM, measured fastest for 144 components).  Each block keeps Wb transposed
// (C x kMaxBasis, zero-padded) in shared memory and two feature-tile buffers (row
// stride C + 4 words) filled by 16-byte asynchronous copies issued two tiles
// ahead, so the loads of the next tile overlap the arithmetic of this one.
// Product: thread t owns columns 4 (t % 8) .. +3 of rows t / 8 + (NT / 8) i, i <
// RPT; per 4 inputs it reads one float4 of each of its rows and four
// float4 weight rows (the four rows a warp touches fall in distinct banks) and
// accumulates with packed two-lane FMAs (the same rounding as scalar FMAs, in
// the same order).  Encoding: B goes through shared memory and a warp takes two
// rows at a time, lane f feature f (lanes F .. F + 2 the view direction): one
// sincos16 of the value, the 2^k multiples by the double-angle recurrence
// sin 2a = 2 sin a cos a, cos 2a = (cos a - sin a)(cos a + sin a) (fp32 error
// ~ 2^k ulp, far below the 16-bit rounding of the output), written into the
// consumed tile buffer as the 16-bit staging (row stride k1p + 8), which the
// block stores as 16-byte vectors.

// (d0, d1) += a * (b0, b1) with one packed two-lane FMA (fma.rn per lane)
__device__ __forceinline__ void ffma2(float& d0, float& d1, float a, float b0, float b1) {
    const float2 r = __ffma2_rn(make_float2(a, a), make_float2(b0, b1), make_float2(d0, d1));
    d0 = r.x;
    d1 = r.y;
}

// sin and cos of x for the 16-bit encodings: x = k pi/2 + r, k = rint(x 2/pi), r
// reduced with the two-term Cody-Waite split pi/2 = kPio2Hi + kPio2Lo (the first
// product exact inside an FMA), |r| <= pi/4, then the hardware approximations on r
// and the quadrant k mod 4.  Absolute error ~5e-7 (far below 16-bit rounding);
// sincosf beyond |x| = 1e5, where k no longer fits the reduction's precision.
constexpr float kPio2Hi = 1.57079637050628662109375f;        // pi/2 rounded to float
constexpr float kPio2Lo = -4.37113900018624283e-8f;          // pi/2 - kPio2Hi
__device__ __forceinline__ void sincos16(float x, float* s, float* c) {
    if (!(fabsf(x) <= 1e5f)) {
        sincosf(x, s, c);
        return;
    }
    const float k = rintf(x * 0.636619772367581343f);
    const float r = fmaf(-k, kPio2Lo, fmaf(-k, kPio2Hi, x));
    const float sr = __sinf(r), cr = __cosf(r);
    const int q = int(k) & 3;
    *s = (q & 1) ? ((q & 2) ? -cr : cr) : ((q & 2) ? -sr : sr);
    *c = (q & 1) ? ((q & 2) ? sr : -sr) : ((q & 2) ? -cr : cr);
}

// (d0, d1) += (a0, a1) * (b0, b1) with one packed two-lane FMA
__device__ __forceinline__ void fma2v(float& d0, float& d1, float a0, float a1, float b0, float b1) {
    const float2 r = __ffma2_rn(make_float2(a0, a1), make_float2(b0, b1), make_float2(d0, d1));
    d0 = r.x;
    d1 = r.y;
}

__host__ __device__ inline int enc_tile_rows(int rpt, int nt) { return nt / 8 * rpt; }
constexpr int kEncBStride = kMaxBasis + 1;   // row stride (words) of the B tile in shared memory
// the 16-bit staging rows of a tile (16-byte multiple), followed by its B rows
__host__ __device__ inline size_t enc_stage_bytes(int k1p, int rpt, int nt) {
    return size_t(enc_tile_rows(rpt, nt)) * (k1p + 8) * sizeof(op16);
}
__host__ __device__ inline size_t enc_buf_bytes(int C, int k1p, int rpt, int nt) {
    size_t fb = size_t(enc_tile_rows(rpt, nt)) * (C + 4) * sizeof(float);
    size_t xb = enc_stage_bytes(k1p, rpt, nt) + size_t(enc_tile_rows(rpt, nt)) * kEncBStride * sizeof(float);
    const size_t m = fb > xb ? fb : xb;
    return (m + 15) / 16 * 16;
}
__host__ __device__ inline size_t enc_smem_bytes(int C, int k1p, int rpt, int nt) {
    return size_t(C) * kMaxBasis * sizeof(float) + 2 * enc_buf_bytes(C, k1p, rpt, nt);
}

// WbT[c, o] = Wb[o, c] for o < F, 0 up to kMaxBasis: the layout the basis pass
// loads with 128-bit reads (one per-step pass over F x C weights).
__global__ void transpose_basis_kernel(const float* __restrict__ Wb, int F, int C, float* WbT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C * kMaxBasis) return;
    const int c = i / kMaxBasis, o = i - c * kMaxBasis;
    WbT[i] = o < F ? Wb[o * C + c] : 0.f;
}

template <int RPT, int NT>
__global__ void __launch_bounds__(NT)
    basis_encode_kernel(const float* __restrict__ feats, int C, const float* __restrict__ WbT, int F,
                        const float* __restrict__ view, int64_t M, int lf, int lv, int bw, int bs, int k1p, float* B,
                        op16* x, int fmt) {
    extern __shared__ __align__(16) float esm[];
    constexpr int RG = NT / 8, T = RG * RPT;                   // row groups, rows per tile
    float* sWt = esm;                                          // C x kMaxBasis
    const size_t buf_words = enc_buf_bytes(C, k1p, RPT, NT) / sizeof(float);
    float* bufs = esm + size_t(C) * kMaxBasis;
    const int S = C + 4, XS = k1p + 8;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t ntiles = (M + T - 1) / T;
    {
        const float4* src = reinterpret_cast<const float4*>(WbT);
        float4* dst = reinterpret_cast<float4*>(sWt);
        for (int i = tid; i < C * kMaxBasis / 4; i += NT) dst[i] = src[i];
    }
    // asynchronous copy of tile t's feature rows into buffer b (nothing past the last tile)
    auto issue = [&](int64_t t, int b) {
        if (t < ntiles) {
            const int64_t r0 = t * T;
            const int rows = M - r0 < T ? int(M - r0) : T;
            float* dst = bufs + b * buf_words;
            for (int r = warp; r < rows; r += NT / 32) {
                const float* g = feats + (r0 + r) * C;
                for (int q = lane; q < C / 4; q += 32) cp_async16(dst + r * S + 4 * q, g + 4 * q);
            }
        }
        cp_async_commit();
    };
    int64_t tile = blockIdx.x;
    issue(tile, 0);
    issue(tile + gridDim.x, 1);
    const int rg = tid >> 3, cg = tid & 7;
    const float4* w4 = reinterpret_cast<const float4*>(sWt) + cg;   // + c * (kMaxBasis / 4)
    for (int k = 0; tile < ntiles; ++k, tile += gridDim.x) {
        const int b = k & 1;
        float* buf = bufs + b * buf_words;
        const int64_t row0 = tile * T;
        const int rows = M - row0 < T ? int(M - row0) : T;
        cp_async_wait_one();
        __syncthreads();
        float2 acc[RPT][2];
#pragma unroll
        for (int i = 0; i < RPT; ++i) acc[i][0] = acc[i][1] = make_float2(0.f, 0.f);
        const float* f0 = buf + rg * S;
        for (int c = 0; c < C; c += 4) {
            const float4 wa = w4[(c + 0) * (kMaxBasis / 4)], wb = w4[(c + 1) * (kMaxBasis / 4)];
            const float4 wc = w4[(c + 2) * (kMaxBasis / 4)], wd = w4[(c + 3) * (kMaxBasis / 4)];
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                const float4 f = *reinterpret_cast<const float4*>(f0 + RG * i * S + c);
                const float2 fx = make_float2(f.x, f.x), fy = make_float2(f.y, f.y);
                const float2 fz = make_float2(f.z, f.z), fw = make_float2(f.w, f.w);
                acc[i][0] = __ffma2_rn(fx, make_float2(wa.x, wa.y), acc[i][0]);
                acc[i][1] = __ffma2_rn(fx, make_float2(wa.z, wa.w), acc[i][1]);
                acc[i][0] = __ffma2_rn(fy, make_float2(wb.x, wb.y), acc[i][0]);
                acc[i][1] = __ffma2_rn(fy, make_float2(wb.z, wb.w), acc[i][1]);
                acc[i][0] = __ffma2_rn(fz, make_float2(wc.x, wc.y), acc[i][0]);
                acc[i][1] = __ffma2_rn(fz, make_float2(wc.z, wc.w), acc[i][1]);
                acc[i][0] = __ffma2_rn(fw, make_float2(wd.x, wd.y), acc[i][0]);
                acc[i][1] = __ffma2_rn(fw, make_float2(wd.z, wd.w), acc[i][1]);
            }
        }
        __syncthreads();   // the tile buffer becomes the staging + B tile
        op16* stage = reinterpret_cast<op16*>(buf);
        float* sB = reinterpret_cast<float*>(reinterpret_cast<uint8_t*>(buf) + enc_stage_bytes(k1p, RPT, NT));
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
            float* d = sB + (rg + RG * i) * kEncBStride + cg * 4;
            d[0] = acc[i][0].x;
            d[1] = acc[i][0].y;
            d[2] = acc[i][1].x;
            d[3] = acc[i][1].y;
        }
        __syncthreads();
        // every staged row starts as zeros (the gaps after each block and the tail)
        for (int r = warp; r < rows; r += NT / 32) {
            uint32_t* my = reinterpret_cast<uint32_t*>(stage + r * XS);
            for (int c = lane; c < k1p / 2; c += 32) my[c] = 0u;
        }
        __syncwarp();
        // lane roles: feature f = lane (f < F), view component a (lanes F .. F + 2, or a
        // second pass on lanes 0 .. 2 when F > 29); each writes its value, then sin and
        // cos of 2^q value at columns c_sin + q dq and c_sin + q dq + dcos
        const int v0 = bw * (2 * lf + 1);
        const bool view_here = view && F <= 29;
        for (int pass = 0; pass < ((view && F > 29) ? 2 : 1); ++pass) {
            int kind = 0, col = 0, csin = 0, dq = 0, dcos = 0, deg = 0;   // kind 1: feature, 2: view
            if (pass == 0 && lane < F) {
                kind = 1; col = lane; csin = bw + lane; dq = 2 * bw; dcos = bw; deg = lf;
            } else if (view && ((pass == 0 && view_here && lane >= F && lane < F + 3) || (pass == 1 && lane < 3))) {
                const int a = pass == 0 ? lane - F : lane;
                kind = 2; col = v0 + a; csin = v0 + 3 + a; dq = 6; dcos = 3; deg = lv;
            }
            const int a_view = col - v0;
            for (int r0 = warp; r0 < rows; r0 += 2 * (NT / 32)) {
                const int r1 = r0 + NT / 32;
                const bool two = r1 < rows;
                float v[2] = {0.f, 0.f};
                if (kind == 1) {
                    v[0] = sB[r0 * kEncBStride + lane];
                    if (two) v[1] = sB[r1 * kEncBStride + lane];
                } else if (kind == 2) {
                    v[0] = view[(row0 + r0) * 3 + a_view];
                    if (two) v[1] = view[(row0 + r1) * 3 + a_view];
                }
                float sn[2], cs[2];
                sincos16(v[0], &sn[0], &cs[0]);
                sincos16(v[1], &sn[1], &cs[1]);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int r = h ? r1 : r0;
                    if (kind == 0 || (h && !two)) continue;
                    op16* my = stage + r * XS;
                    if (kind == 1) B[(row0 + r) * bs + lane] = v[h];
                    my[col] = tc::to16(v[h], fmt);
                    float sh = sn[h], ch = cs[h];
                    for (int q = 0; q < deg; ++q) {
                        my[csin + q * dq] = tc::to16(sh, fmt);
                        my[csin + q * dq + dcos] = tc::to16(ch, fmt);
                        const float s2 = 2.f * sh * ch, c2 = (ch - sh) * (ch + sh);
                        sh = s2;
                        ch = c2;
                    }
                }
            }
        }
        __syncthreads();
        {
            const int nq = k1p / 8;
            for (int r = warp; r < rows; r += NT / 32) {
                const uint4* src = reinterpret_cast<const uint4*>(stage + r * XS);
                uint4* dst = reinterpret_cast<uint4*>(x + (row0 + r) * k1p);
                for (int q = lane; q < nq; q += 32) dst[q] = src[q];
            }
        }
        __syncthreads();   // staging consumed: the buffer takes tile + 2 grid
        issue(tile + 2 * int64_t(gridDim.x), b);
    }
    cp_async_wait_all();
}

// Basis-layer backward fused with the PE adjoint, over a contiguous range of rows
// per block, kBwdTile rows at a time:
//   dB[m, o]    = sum over the PE columns of B[m, o] of dx * d(column)/dB (dx: the
//                 16-bit encoded-row gradient, loss-scaled by gscale[0]; unscaled here)
//   d_feats[m]  = dB[m] . Wb                       (written)
//   dWb        += dB^T . feats                     (one atomic per weight per block)
// The feature, dx and B rows of each tile arrive in shared memory by asynchronous
// copies issued one tile ahead (two buffers), so the loads of tile t + 1 overlap
// the arithmetic of tile t.  Thread c owns feature column c, with its Wb column
// and its dWb accumulators in registers; dB rows are shared-memory broadcasts.
constexpr int kBwdTile = 32;

// shared bytes of one tile buffer: feature rows, dx rows, B rows (bs floats each)
__host__ __device__ inline size_t basis_tile_bytes(int C, int bs, int k1p) {
    return size_t(kBwdTile) * C * 4 + size_t(kBwdTile) * k1p * 2 + size_t(kBwdTile) * bs * 4;
}
__host__ __device__ inline size_t basis_bwd_smem(int C, int bs, int k1p) {
    return size_t(kBwdTile) * kMaxBasis * 4 + 2 * basis_tile_bytes(C, bs, k1p);
}

__global__ void basis_bwd_kernel(const op16* __restrict__ dx, const float* __restrict__ B,
                                 const float* __restrict__ feats, const float* __restrict__ Wb, int64_t M, int F,
                                 int C, int lf, int bw, int bs, int k1p, int fmt, const float* gscale,
                                 int64_t rows_per_block, float* d_feats, float* dWb) {
    extern __shared__ __align__(16) float bb[];
    float* sdB = bb;                                   // kBwdTile x kMaxBasis
    uint8_t* bufs = reinterpret_cast<uint8_t*>(sdB + kBwdTile * kMaxBasis);
    const size_t tile_bytes = basis_tile_bytes(C, bs, k1p);
    const float unscale = gscale ? gscale[1] : 1.f;
    const int c = threadIdx.x;
    float wcol[kMaxBasis], acc[kMaxBasis];
#pragma unroll
    for (int o = 0; o < kMaxBasis; ++o) {
        wcol[o] = (c < C && o < F) ? Wb[o * C + c] : 0.f;
        acc[o] = 0.f;
    }
    const int64_t r_begin = int64_t(blockIdx.x) * rows_per_block;
    const int64_t r_end = r_begin + rows_per_block < M ? r_begin + rows_per_block : M;
    // issue the asynchronous copies of the tile at row t0 into buffer `which`
    auto load_tile = [&](int64_t t0, int which) {
        if (t0 < r_end) {
            const int nt = int(r_end - t0 < kBwdTile ? r_end - t0 : kBwdTile);
            uint8_t* base = bufs + which * tile_bytes;
            float* sF = reinterpret_cast<float*>(base);
            op16* sdx = reinterpret_cast<op16*>(base + size_t(kBwdTile) * C * 4);
            float* sB = reinterpret_cast<float*>(base + size_t(kBwdTile) * C * 4 + size_t(kBwdTile) * k1p * 2);
            const float* gf = feats + t0 * C;          // rows are contiguous: nt * C floats
            for (int i = threadIdx.x; i < nt * C / 4; i += blockDim.x) cp_async16(sF + 4 * i, gf + 4 * i);
            const op16* gx = dx + t0 * k1p;
            for (int i = threadIdx.x; i < nt * k1p / 8; i += blockDim.x) cp_async16(sdx + 8 * i, gx + 8 * i);
            const float* gb = B + t0 * bs;   // bs is a multiple of 4 floats
            for (int i = threadIdx.x; i < nt * bs / 4; i += blockDim.x) cp_async16(sB + 4 * i, gb + 4 * i);
        }
        cp_async_commit();
    };
    load_tile(r_begin, 0);
    int buf = 0;
    for (int64_t t0 = r_begin; t0 < r_end; t0 += kBwdTile, buf ^= 1) {
        const int nt = int(r_end - t0 < kBwdTile ? r_end - t0 : kBwdTile);
        load_tile(t0 + kBwdTile, buf ^ 1);   // the next tile streams in under this one
        cp_async_wait_one();
        __syncthreads();
        uint8_t* base = bufs + buf * tile_bytes;
        const float* sF = reinterpret_cast<const float*>(base);
        const op16* sdx = reinterpret_cast<const op16*>(base + size_t(kBwdTile) * C * 4);
        const float* sB = reinterpret_cast<const float*>(base + size_t(kBwdTile) * C * 4 + size_t(kBwdTile) * k1p * 2);
        for (int i = threadIdx.x; i < kBwdTile * kMaxBasis; i += blockDim.x) {
            const int rr = i / kMaxBasis, o = i - rr * kMaxBasis;
            float g = 0.f;
            if (rr < nt && o < F) {
                const op16* row = sdx + rr * k1p;
                auto rd = [&](int col) {
                    const uint32_t w = reinterpret_cast<const uint32_t*>(row)[col >> 1];
                    const float2 f = tc::unpack16(w, fmt);
                    return (col & 1) ? f.y : f.x;
                };
                const float bo = sB[rr * bs + o];
                g = rd(o);
                float sn, cs;   // sin, cos of 2^k B by the double-angle recurrence
                sincos16(bo, &sn, &cs);
                for (int k = 0; k < lf; ++k) {
                    const float fk = float(1 << k);
                    g += fk * (cs * rd((2 * k + 1) * bw + o) - sn * rd((2 * k + 2) * bw + o));
                    const float s2 = 2.f * sn * cs, c2 = (cs - sn) * (cs + sn);
                    sn = s2;
                    cs = c2;
                }
                g *= unscale;
            }
            sdB[i] = g;
        }
        __syncthreads();
        if (c < C) {
            // two rows per pass: their dB . Wb chains are independent (the dWb
            // accumulators still take the rows in order)
            int rr = 0;
            for (; rr + 1 < nt; rr += 2) {
                const float f0 = sF[rr * C + c], f1 = sF[(rr + 1) * C + c];
                float de0 = 0.f, dd0 = 0.f, de1 = 0.f, dd1 = 0.f;   // even / odd basis columns of dB . Wb
#pragma unroll
                for (int o4 = 0; o4 < kMaxBasis; o4 += 4) {
                    if (o4 >= F) break;
                    const float4 d0 = *reinterpret_cast<const float4*>(sdB + rr * kMaxBasis + o4);
                    const float4 d1 = *reinterpret_cast<const float4*>(sdB + (rr + 1) * kMaxBasis + o4);
                    fma2v(de0, dd0, d0.x, d0.y, wcol[o4], wcol[o4 + 1]);
                    fma2v(de1, dd1, d1.x, d1.y, wcol[o4], wcol[o4 + 1]);
                    fma2v(de0, dd0, d0.z, d0.w, wcol[o4 + 2], wcol[o4 + 3]);
                    fma2v(de1, dd1, d1.z, d1.w, wcol[o4 + 2], wcol[o4 + 3]);
                    ffma2(acc[o4], acc[o4 + 1], f0, d0.x, d0.y);
                    ffma2(acc[o4 + 2], acc[o4 + 3], f0, d0.z, d0.w);
                    ffma2(acc[o4], acc[o4 + 1], f1, d1.x, d1.y);
                    ffma2(acc[o4 + 2], acc[o4 + 3], f1, d1.z, d1.w);
                }
                d_feats[(t0 + rr) * C + c] = de0 + dd0;
                d_feats[(t0 + rr + 1) * C + c] = de1 + dd1;
            }
            for (; rr < nt; ++rr) {
                const float f = sF[rr * C + c];
                float de = 0.f, dd = 0.f;
#pragma unroll
                for (int o4 = 0; o4 < kMaxBasis; o4 += 4) {
                    if (o4 >= F) break;
                    const float4 d = *reinterpret_cast<const float4*>(sdB + rr * kMaxBasis + o4);
                    fma2v(de, dd, d.x, d.y, wcol[o4], wcol[o4 + 1]);
                    fma2v(de, dd, d.z, d.w, wcol[o4 + 2], wcol[o4 + 3]);
                    ffma2(acc[o4], acc[o4 + 1], f, d.x, d.y);
                    ffma2(acc[o4 + 2], acc[o4 + 3], f, d.z, d.w);
                }
                d_feats[(t0 + rr) * C + c] = de + dd;
            }
        }
        __syncthreads();   // buffer `buf` and sdB are rewritten next round
    }
    cp_async_wait_all();
    if (c < C) {
#pragma unroll
        for (int o = 0; o < kMaxBasis; ++o)
            if (o < F) atomicAdd(dWb + o * C + c, acc[o]);
    }
}

}  // namespace

size_t render_tc_workspace(int C, int F, int U, int lf, int lv, int view, int64_t m, bool bwd) {
    RenderLayout R(C, F, U, lf, lv, view);
    if (!R.ok) return 0;
    return carve_render(R, m, bwd, nullptr, ~size_t(0), nullptr);
}

template <int RPT, int NT>
int launch_basis_encode_cfg(const float* feats, int C, const float* WbT, int F, const float* view, int64_t m, int lf,
                            int lv, int bw, int bs, int k1p, float* B, op16* x, int fmt, cudaStream_t s) {
    const size_t smem = enc_smem_bytes(C, k1p, RPT, NT);
    cudaError_t e = cudaFuncSetAttribute(basis_encode_kernel<RPT, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(smem));
    int per_sm = 0;
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, basis_encode_kernel<RPT, NT>, NT, smem);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return SRF_ERR_CUDA;
    }
    const int64_t tiles = (m + enc_tile_rows(RPT, NT) - 1) / enc_tile_rows(RPT, NT);
    int64_t grid = int64_t(num_sms()) * (per_sm > 0 ? per_sm : 1);
    if (grid > tiles) grid = tiles;
    basis_encode_kernel<RPT, NT><<<unsigned(grid), NT, smem, s>>>(feats, C, WbT, F, view, m, lf, lv, bw, bs, k1p, B,
                                                                  x, fmt);
    return launch_status();
}

// ---------------------------------------------------------------------------
// The basis pass on the tensor cores: B = feats . Wb^T as a TF32 tcgen05 GEMM
// (128 sample rows per tile, N = 32 >= F basis outputs, K = C components in
// 32-float blocks loaded by TMA with the 128-byte swizzle; components past C and
// basis rows past F read as zeros), the positional encoding of B and of the view
// direction in the epilogue.  Same outputs and layout as basis_encode_kernel (B
// rows of kMaxBasis floats, x in RenderLayout's blocked columns).  The TF32
// products round feats and Wb to 10 mantissa bits (relative error ~5e-4), below
// the 16-bit rounding of x they feed.
// Warp roles (320 threads, one CTA per SM, persistent over tiles): warp 0 issues
// the TMA loads (Wb once, then a ring of feature blocks), warp 1 the MMAs into
// four 32-column tensor-memory accumulators, warps 2..9 in two groups of four
// that take alternate tiles, each warp of a group reading one lane quadrant (a
// thread per row).  A thread encodes its row eight columns at a time and
// writes each 16-byte piece into its warp's staging boxes in the 128-byte
// swizzled layout (the eight rows of a quarter-warp land in eight distinct bank
// groups); lane 0 then stores the boxes with TMA (x in 64-column boxes, B in one
// 32-float box) while the warp moves on to its next tile.  Every mbarrier wait
// is bounded as in the layer GEMM.
namespace {

constexpr int kBtMaxStages = 6;
constexpr int kBtEpiWarps = 8;             // two groups of four
constexpr int kBtThreads = 64 + 32 * kBtEpiWarps;
constexpr uint32_t kBtATile = 128 * 128;   // 128 rows x 32 floats
constexpr uint32_t kBtBBlock = 32 * 128;   // 32 rows x 32 floats
constexpr uint32_t kBtBox = 32 * 128;      // a staging box: 32 rows x 128 bytes

__host__ __device__ inline int bt_kblocks(int C) { return (C + 31) / 32; }
__host__ __device__ inline size_t bt_stage_bytes(int k1p) { return size_t(k1p / 64 + 1) * kBtBox; }
__host__ __device__ inline size_t bt_fixed_smem(int C, int k1p) {
    return 1024 + size_t(bt_kblocks(C)) * kBtBBlock + kBtEpiWarps * bt_stage_bytes(k1p) + 256;
}
// feature-block ring stages that fit beside the fixed parts (0 or 1: the pass does not fit)
inline int bt_stages(int C, int k1p) {
    const size_t fixed = bt_fixed_smem(C, k1p);
    if (fixed >= tc::kMaxSmem) return 0;
    const size_t st = (tc::kMaxSmem - fixed) / kBtATile;
    return int(st < size_t(kBtMaxStages) ? st : size_t(kBtMaxStages));
}
inline size_t bt_smem(int C, int k1p, int stages) { return bt_fixed_smem(C, k1p) + size_t(stages) * kBtATile; }

// Instruction descriptor of kind::tf32: F32 accumulator (bits 4-5 = 1), A and B
// TF32 (format 2 at bits 7-9 and 10-12), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t idesc_tf32(int m, int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(m >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// 2-D map of `dtype` elements: `inner` contiguous elements per row, `outer` rows of
// `row_bytes`, boxes of box_in x box_out with the 128-byte swizzle.
bool make_map_t(CUtensorMap* m, CUtensorMapDataType dtype, const void* ptr, uint64_t inner, uint64_t outer,
                uint64_t row_bytes, uint32_t box_in, uint32_t box_out) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {row_bytes};
    cuuint32_t box[2] = {box_in, box_out};
    cuuint32_t es[2] = {1, 1};
    return fn(m, dtype, 2, const_cast<void*>(ptr), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Eight floats -> eight 16-bit words of format FMT; entries at and past `valid` as zeros.
template <int FMT>
__device__ __forceinline__ uint4 pack8(const float* a, int valid) {
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = i < valid ? a[i] : 0.f;
    return make_uint4(tc::pack16(v[0], v[1], FMT), tc::pack16(v[2], v[3], FMT), tc::pack16(v[4], v[5], FMT),
                      tc::pack16(v[6], v[7], FMT));
}

template <int FMT>
__global__ void __launch_bounds__(kBtThreads, 1)
    basis_tc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmW,
                    const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmB, int64_t M,
                    int C, int F, const float* __restrict__ view, int lf, int lv, int bw, int k1p, int stages,
                    int* flag) {
    using namespace tc;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int KB = bt_kblocks(C);
    const int nbx = k1p / 64;   // 64-column x boxes per row group
    uint8_t* sW = base;
    uint8_t* sA = sW + size_t(KB) * kBtBBlock;
    uint8_t* sStage = sA + size_t(stages) * kBtATile;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sStage + kBtEpiWarps * bt_stage_bytes(k1p));
    uint64_t* full = bars;                          // [kBtMaxStages]
    uint64_t* empty = bars + kBtMaxStages;          // [kBtMaxStages]
    uint64_t* acc_full = bars + 2 * kBtMaxStages;   // [4]
    uint64_t* acc_empty = acc_full + 4;             // [4]
    uint64_t* w_full = acc_empty + 4;
    uint64_t* done = w_full + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t num_tiles = (M + 127) / 128;
    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 4; ++a) {
            mbar_init(&acc_full[a], 1);
            mbar_init(&acc_empty[a], 128);
        }
        mbar_init(w_full, 1);
        mbar_init(done, 1);
        *abort_flag = 0;
        fence_barrier_init();
    }
    if (warp == 1) {
        tmem_alloc(tmem_slot, 128);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ------------------------------------------------------------ producer
        prefetch_tmap(&tmA);
        prefetch_tmap(&tmW);
        mbar_arrive_expect_tx(w_full, uint32_t(KB) * kBtBBlock);
        for (int kb = 0; kb < KB; ++kb) tma_load_2d(sW + size_t(kb) * kBtBBlock, &tmW, w_full, kb * 32, 0);
        uint32_t it = 0;
        uint32_t last_parity[kBtMaxStages] = {};
        bool used[kBtMaxStages] = {};
        for (int64_t tile = blockIdx.x; tile < num_tiles && !*abort_flag; tile += gridDim.x) {
            for (int kb = 0; kb < KB; ++kb, ++it) {
                const int s = int(it % uint32_t(stages));
                const uint32_t ph = (it / uint32_t(stages)) & 1;
                if (!mbar_wait(&empty[s], ph ^ 1, abort_flag)) {
                    *abort_flag = 1;
                    break;
                }
                mbar_arrive_expect_tx(&full[s], kBtATile);
                tma_load_2d(sA + size_t(s) * kBtATile, &tmA, &full[s], kb * 32, int32_t(tile * 128));
                used[s] = true;
                last_parity[s] = ph;
            }
        }
        // every copy this thread started has landed before the CTA may exit
        for (int s = 0; s < stages; ++s)
            if (used[s] && !mbar_wait(&full[s], last_parity[s], nullptr)) *abort_flag = 1;
        if (!mbar_wait(w_full, 0, nullptr)) *abort_flag = 1;
    } else if (warp == 1 && lane == 0) {
        // ---------------------------------------------------------------- MMA
        const uint32_t idesc = idesc_tf32(128, 32);
        bool ok = mbar_wait(w_full, 0, abort_flag);
        uint32_t it = 0, t = 0;
        for (int64_t tile = blockIdx.x; ok && tile < num_tiles; tile += gridDim.x, ++t) {
            const uint32_t acc = t & 3;
            if (!mbar_wait(&acc_empty[acc], ((t >> 2) & 1) ^ 1, abort_flag)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t d_tmem = tmem + acc * 32;
            for (int kb = 0; kb < KB; ++kb, ++it) {
                const int s = int(it % uint32_t(stages));
                if (!mbar_wait(&full[s], (it / uint32_t(stages)) & 1, abort_flag)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t a_addr = smem_u32(sA + size_t(s) * kBtATile);
                const uint32_t b_addr = smem_u32(sW + size_t(kb) * kBtBBlock);
#pragma unroll
                for (int k = 0; k < 4; ++k) {   // K = 8 TF32 values (32 bytes) per MMA
                    const uint64_t ad = smem_desc(a_addr + k * 32, 0, 1024, kSwizzle128B);
                    const uint64_t bd = smem_desc(b_addr + k * 32, 0, 1024, kSwizzle128B);
                    mma_tf32(d_tmem, ad, bd, idesc, (kb | k) != 0);
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
        // ----------------------------------------------------------- epilogue
        const int q = warp & 3;           // the tensor-memory lane quadrant this warp may read
        const int grp = (warp - 2) >> 2;  // group 0 takes the CTA's even tiles, group 1 the odd
        uint8_t* stX = sStage + size_t(warp - 2) * bt_stage_bytes(k1p);   // nbx boxes, then the B box
        uint8_t* stB = stX + size_t(nbx) * kBtBox;
        const uint32_t rowoff = uint32_t(lane) * 128u, sw = uint32_t(lane & 7);
        // 16-byte piece j (columns 8 j .. 8 j + 7) of this thread's x row
        auto put_x = [&](int j, uint4 v) {
            *reinterpret_cast<uint4*>(stX + size_t(j >> 3) * kBtBox + rowoff + ((uint32_t(j & 7) ^ sw) << 4)) = v;
        };
        const int fb = bw / 8, vp0 = (2 * lf + 1) * fb, np = k1p / 8;
        const float zero8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (uint32_t t = uint32_t(grp);; t += 2) {
            const int64_t tile = blockIdx.x + int64_t(t) * gridDim.x;
            if (tile >= num_tiles) break;
            const uint32_t acc = t & 3;
            const int64_t row0 = tile * 128 + q * 32;
            const int64_t m = row0 + lane;
            float dv[3] = {0.f, 0.f, 0.f};
            if (view && m < M) {
                dv[0] = view[m * 3];
                dv[1] = view[m * 3 + 1];
                dv[2] = view[m * 3 + 2];
            }
            if (!mbar_wait(&acc_full[acc], (t >> 2) & 1, abort_flag)) {
                *abort_flag = 1;
                break;
            }
            tc_fence_after();
            uint32_t r[32];
            tmem_ld_32x32b_x32(tmem + acc * 32 + (uint32_t(q * 32) << 16), r);
            tmem_ld_wait();
            tc_fence_before();
            mbar_arrive(&acc_empty[acc]);
            // the previous tile's stores have finished reading the staging boxes
            if (lane == 0) bulk_wait_read_all();
            __syncwarp();
            // B row: columns past F are zeros (Wb rows past F read as zeros)
#pragma unroll
            for (int j = 0; j < 8; ++j)
                *reinterpret_cast<uint4*>(stB + rowoff + ((uint32_t(j) ^ sw) << 4)) =
                    make_uint4(r[4 * j], r[4 * j + 1], r[4 * j + 2], r[4 * j + 3]);
            // feature blocks, eight features at a time: B, then sin / cos of 2^k B
#pragma unroll
            for (int g = 0; g < kMaxBasis / 8; ++g) {
                if (g < fb) {
                    const int valid = F - 8 * g;
                    float sn[8], cs[8], v[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        v[i] = __uint_as_float(r[8 * g + i]);
                        sincos16(v[i], &sn[i], &cs[i]);
                    }
                    put_x(g, pack8<FMT>(v, valid));
                    for (int k = 0; k < lf; ++k) {
                        put_x((2 * k + 1) * fb + g, pack8<FMT>(sn, valid));
                        put_x((2 * k + 2) * fb + g, pack8<FMT>(cs, valid));
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            const float s2 = 2.f * sn[i] * cs[i], c2 = (cs[i] - sn[i]) * (cs[i] + sn[i]);
                            sn[i] = s2;
                            cs[i] = c2;
                        }
                    }
                }
            }
            // view block [d, sin d, cos d, sin 2d, cos 2d, ...] (lv <= 4: at most 27
            // values, four pieces), zeros up to k1p
            float vv[32];
#pragma unroll
            for (int i = 0; i < 32; ++i) vv[i] = 0.f;
            if (view) {
                float sn[3], cs[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    vv[a] = dv[a];
                    sincos16(dv[a], &sn[a], &cs[a]);
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (k < lv) {
#pragma unroll
                        for (int a = 0; a < 3; ++a) {
                            vv[3 + 6 * k + a] = sn[a];
                            vv[6 + 6 * k + a] = cs[a];
                            const float s2 = 2.f * sn[a] * cs[a], c2 = (cs[a] - sn[a]) * (cs[a] + sn[a]);
                            sn[a] = s2;
                            cs[a] = c2;
                        }
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (vp0 + j < np) put_x(vp0 + j, pack8<FMT>(vv + 8 * j, 8));
            for (int j = vp0 + 4; j < np; ++j) put_x(j, pack8<FMT>(zero8, 0));
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0 && row0 < M) {
                for (int b = 0; b < nbx; ++b) tma_store_2d(&tmX, stX + size_t(b) * kBtBox, b * 64, int32_t(row0));
                tma_store_2d(&tmB, stB, 0, int32_t(row0));
                bulk_commit_group();
            }
        }
        if (lane == 0) bulk_wait_all();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 128);
    }
    if (threadIdx.x == 0 && *abort_flag) raise_flag(flag, kFlagTimeout);
}

// The basis adjoint on the tensor cores, for the rows of one backward call:
//   dB[m, o]   = (1 / loss scale) sum over the PE columns of B[m, o] of dx * d(column)/dB
//   d_feats[m] = dB[m] . Wb              (TF32 tcgen05 GEMM, M = 128 rows, N = C, K = 32)
// and dB itself written out for basis_wgrad_kernel (dWb += dB^T feats).
// Warp roles (320 threads, one CTA per SM, persistent over tiles): warp 0 streams
// each tile's dx (64-column boxes) and B rows through a two-stage TMA ring and
// loads WbT (C x 32, the B operand, K-major) once; warps 2..9, two groups of four
// taking alternate tiles (group g the ring stage g and dB tile g), form dB, a
// thread per row, from the swizzled dx and B rows, write it as the MMA's A tile
// (128 x 32 floats, 128-byte swizzle) and store their 32 rows of it with TMA; warp
// 1 issues the four K = 8 MMAs per tile into one of two 256-column accumulators;
// warps 10..13 read their lane quadrant of the accumulator (a thread per row) and
// store the d_feats rows with 16-byte stores.  Every mbarrier wait is bounded.
constexpr int kBbThreads = 448;
constexpr uint32_t kBbBox = 128 * 128;       // a 128-row x 128-byte box (dx or B rows)

__host__ __device__ inline size_t bb_stage_bytes(int k1p) { return size_t(k1p / 64 + 1) * kBbBox; }
__host__ __device__ inline size_t bb_smem(int C, int k1p) {
    return 1024 + size_t((C + 7) / 8 * 8) * 128 + 2 * bb_stage_bytes(k1p) + 2 * size_t(kBbBox) + 256;
}

__global__ void __launch_bounds__(kBbThreads, 1)
    basis_bwd_tc_kernel(const __grid_constant__ CUtensorMap tmDX, const __grid_constant__ CUtensorMap tmB,
                        const __grid_constant__ CUtensorMap tmWT, const __grid_constant__ CUtensorMap tmDB,
                        int64_t M, int C, int F, int lf, int bw, int k1p, int fmt, const float* gscale,
                        float* __restrict__ d_feats, int* flag) {
    using namespace tc;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int nbx = k1p / 64;
    const uint32_t wt_bytes = uint32_t((C + 7) / 8 * 8) * 128u;
    uint8_t* sWT = base;
    uint8_t* sRing = sWT + wt_bytes;                        // 2 stages: nbx dx boxes, then the B box
    uint8_t* sA = sRing + 2 * bb_stage_bytes(k1p);          // 2 dB tiles
    uint64_t* bars = reinterpret_cast<uint64_t*>(sA + 2 * size_t(kBbBox));
    uint64_t* full = bars;            // [2] ring stage loaded
    uint64_t* empty = bars + 2;       // [2] ring stage read (128 arrivals)
    uint64_t* a_full = bars + 4;      // [2] dB tile written (128 arrivals)
    uint64_t* a_empty = bars + 6;     // [2] dB tile read by the MMAs
    uint64_t* acc_full = bars + 8;    // [2]
    uint64_t* acc_empty = bars + 10;  // [2] (128 arrivals)
    uint64_t* w_full = bars + 12;
    uint64_t* done = bars + 13;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 14);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t num_tiles = (M + 127) / 128;
    const int64_t my_tiles = blockIdx.x < num_tiles ? (num_tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 128);
            mbar_init(&a_full[i], 128);
            mbar_init(&a_empty[i], 1);
            mbar_init(&acc_full[i], 1);
            mbar_init(&acc_empty[i], 128);
        }
        mbar_init(w_full, 1);
        mbar_init(done, 1);
        *abort_flag = 0;
        fence_barrier_init();
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
        // ------------------------------------------------------------ producer
        prefetch_tmap(&tmDX);
        prefetch_tmap(&tmB);
        prefetch_tmap(&tmWT);
        mbar_arrive_expect_tx(w_full, uint32_t(C) * 128u);
        tma_load_2d(sWT, &tmWT, w_full, 0, 0);
        bool used[2] = {false, false};
        uint32_t last[2] = {0, 0};
        for (int64_t t = 0; t < my_tiles && !*abort_flag; ++t) {
            const int s = int(t & 1);
            const uint32_t ph = uint32_t(t >> 1) & 1;
            if (!mbar_wait(&empty[s], ph ^ 1, abort_flag)) {
                *abort_flag = 1;
                break;
            }
            const int64_t tile = blockIdx.x + t * gridDim.x;
            uint8_t* st = sRing + size_t(s) * bb_stage_bytes(k1p);
            mbar_arrive_expect_tx(&full[s], uint32_t(nbx + 1) * kBbBox);
            for (int j = 0; j < nbx; ++j) tma_load_2d(st + size_t(j) * kBbBox, &tmDX, &full[s], j * 64, int32_t(tile * 128));
            tma_load_2d(st + size_t(nbx) * kBbBox, &tmB, &full[s], 0, int32_t(tile * 128));
            used[s] = true;
            last[s] = ph;
        }
        for (int s = 0; s < 2; ++s)
            if (used[s] && !mbar_wait(&full[s], last[s], nullptr)) *abort_flag = 1;
        if (!mbar_wait(w_full, 0, nullptr)) *abort_flag = 1;
    } else if (warp == 1 && lane == 0) {
        // ---------------------------------------------------------------- MMA
        const uint32_t idesc = idesc_tf32(128, C);
        bool ok = mbar_wait(w_full, 0, abort_flag);
        const uint32_t b_addr = smem_u32(sWT);
        for (int64_t t = 0; ok && t < my_tiles; ++t) {
            const int b = int(t & 1);
            const uint32_t ph = uint32_t(t >> 1) & 1;
            if (!mbar_wait(&acc_empty[b], ph ^ 1, abort_flag) || !mbar_wait(&a_full[b], ph, abort_flag)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t a_addr = smem_u32(sA + size_t(b) * kBbBox);
#pragma unroll
            for (int k = 0; k < 4; ++k) {   // K = 8 TF32 values (32 bytes) per MMA
                const uint64_t ad = smem_desc(a_addr + k * 32, 0, 1024, kSwizzle128B);
                const uint64_t bd = smem_desc(b_addr + k * 32, 0, 1024, kSwizzle128B);
                mma_tf32(tmem + uint32_t(b) * 256u, ad, bd, idesc, k != 0);
            }
            mma_commit(&a_empty[b]);
            mma_commit(&acc_full[b]);
        }
        if (!ok) *abort_flag = 1;
        mma_commit(done);
        if (!mbar_wait(done, 0, nullptr)) *abort_flag = 1;
    } else if (warp >= 2 && warp < 10) {
        // ------------------------------------------------------------- adjoint
        const int grp = (warp - 2) >> 2;        // takes the tiles t with t % 2 == grp
        const int wq = (warp - 2) & 3;          // its 32 rows of the tile
        const int r = wq * 32 + lane;           // row within the tile
        const uint32_t rowoff = uint32_t(r) * 128u, sw = uint32_t(r & 7);
        const float unscale = gscale ? gscale[1] : 1.f;
        const int fb = bw / 8;
        for (int64_t t = grp; t < my_tiles; t += 2) {
            const int s = int(t & 1);
            const uint32_t ph = uint32_t(t >> 1) & 1;
            const int64_t row0 = (blockIdx.x + t * gridDim.x) * 128 + wq * 32;
            if (!mbar_wait(&full[s], ph, abort_flag)) {
                *abort_flag = 1;
                break;
            }
            const uint8_t* st = sRing + size_t(s) * bb_stage_bytes(k1p);
            const uint8_t* sBrow = st + size_t(nbx) * kBbBox + rowoff;
            // 16-byte piece p of this row's dx (eight 16-bit columns) as floats
            auto dx8 = [&](int p, float* o) {
                const uint4 v = *reinterpret_cast<const uint4*>(st + size_t(p >> 3) * kBbBox + rowoff +
                                                                ((uint32_t(p & 7) ^ sw) << 4));
                const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float2 f = unpack16(w[i], fmt);
                    o[2 * i] = f.x;
                    o[2 * i + 1] = f.y;
                }
            };
            float dB[32];
#pragma unroll
            for (int g = 0; g < kMaxBasis / 8; ++g) {
#pragma unroll
                for (int i = 0; i < 8; ++i) dB[8 * g + i] = 0.f;
                if (g < fb) {
                    float bv[8], sn[8], cs[8], acc[8], ds[8], dc[8];
                    const float4 b0 = *reinterpret_cast<const float4*>(sBrow + ((uint32_t(2 * g) ^ sw) << 4));
                    const float4 b1 = *reinterpret_cast<const float4*>(sBrow + ((uint32_t(2 * g + 1) ^ sw) << 4));
                    bv[0] = b0.x; bv[1] = b0.y; bv[2] = b0.z; bv[3] = b0.w;
                    bv[4] = b1.x; bv[5] = b1.y; bv[6] = b1.z; bv[7] = b1.w;
#pragma unroll
                    for (int i = 0; i < 8; ++i)   // B columns past F are not written by every forward
                        if (8 * g + i >= F) bv[i] = 0.f;
                    dx8(g, acc);
#pragma unroll
                    for (int i = 0; i < 8; ++i) sincos16(bv[i], &sn[i], &cs[i]);
                    float fk = 1.f;
                    for (int k = 0; k < lf; ++k) {
                        dx8((2 * k + 1) * fb + g, ds);
                        dx8((2 * k + 2) * fb + g, dc);
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            acc[i] += fk * (cs[i] * ds[i] - sn[i] * dc[i]);
                            const float s2 = 2.f * sn[i] * cs[i], c2 = (cs[i] - sn[i]) * (cs[i] + sn[i]);
                            sn[i] = s2;
                            cs[i] = c2;
                        }
                        fk *= 2.f;
                    }
#pragma unroll
                    for (int i = 0; i < 8; ++i) dB[8 * g + i] = 8 * g + i < F ? acc[i] * unscale : 0.f;
                }
            }
            mbar_arrive(&empty[s]);   // this thread is done with the ring stage
            const int b = int(t & 1);
            if (!mbar_wait(&a_empty[b], ph ^ 1, abort_flag)) {
                *abort_flag = 1;
                break;
            }
            if (lane == 0) bulk_wait_read_all();   // the dB store from this tile buffer has read it
            __syncwarp();
            uint8_t* at = sA + size_t(b) * kBbBox;
#pragma unroll
            for (int j = 0; j < 8; ++j)
                *reinterpret_cast<float4*>(at + rowoff + ((uint32_t(j) ^ sw) << 4)) =
                    make_float4(dB[4 * j], dB[4 * j + 1], dB[4 * j + 2], dB[4 * j + 3]);
            fence_proxy_async_smem();
            mbar_arrive(&a_full[b]);
            __syncwarp();
            if (lane == 0 && row0 < M) {
                tma_store_2d(&tmDB, at + size_t(wq) * 32 * 128, 0, int32_t(row0));
                bulk_commit_group();
            }
        }
        if (lane == 0) bulk_wait_all();
    } else if (warp >= 10) {
        // ----------------------------------------------------------- epilogue
        const int q = warp & 3;   // the tensor-memory lane quadrant this warp may read
        const int nchunk = (C + 31) / 32;
        for (int64_t t = 0; t < my_tiles; ++t) {
            const int b = int(t & 1);
            const uint32_t ph = uint32_t(t >> 1) & 1;
            const int64_t m = (blockIdx.x + t * gridDim.x) * 128 + q * 32 + lane;
            if (!mbar_wait(&acc_full[b], ph, abort_flag)) {
                *abort_flag = 1;
                break;
            }
            tc_fence_after();
            float* dst = d_feats + m * C;
            for (int ch = 0; ch < nchunk; ++ch) {
                uint32_t v[32];
                tmem_ld_32x32b_x32(tmem + uint32_t(b) * 256u + uint32_t(ch * 32) + (uint32_t(q * 32) << 16), v);
                tmem_ld_wait();
                if (m < M) {
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        if (ch * 32 + 4 * j < C)
                            *reinterpret_cast<float4*>(dst + ch * 32 + 4 * j) =
                                make_float4(__uint_as_float(v[4 * j]), __uint_as_float(v[4 * j + 1]),
                                            __uint_as_float(v[4 * j + 2]), __uint_as_float(v[4 * j + 3]));
                }
            }
            tc_fence_before();
            mbar_arrive(&acc_empty[b]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 512);
    }
    if (threadIdx.x == 0 && *abort_flag) raise_flag(flag, kFlagTimeout);
}

// dWb[o, c] += sum over rows of dB[m, o] feats[m, c] (dB rows of 32 floats, zeros
// past F, which the tensor-core adjoint writes), over a contiguous range of rows
// per block in tiles of 32 rows whose feature and dB rows arrive by asynchronous
// copies under the previous tile.  A thread holds a 16-feature x 4-column block of
// dWb in registers (one 128-bit feature load and four 128-bit dB loads feed 64
// FMAs); kWgRowGroups groups of C / 2 threads take interleaved rows of each tile;
// at the end the groups meet in shared memory and the block adds its partial sums
// to dWb atomically.
constexpr int kWgRowGroups = 4;

__global__ void __launch_bounds__(512) basis_wgrad_kernel(const float* __restrict__ dB,
                                                          const float* __restrict__ feats, int64_t M, int F, int C,
                                                          int64_t rows_per_block, float* dWb) {
    extern __shared__ __align__(16) float wsm[];
    const size_t tile_floats = size_t(kBwdTile) * (C + kMaxBasis);
    const int ncg = C / 4, per_rg = 2 * ncg;
    const int rg = threadIdx.x / per_rg, u = threadIdx.x - rg * per_rg;
    const int h = u / ncg, cg = u - h * ncg;   // features 16 h .. 16 h + 15, columns 4 cg .. 4 cg + 3
    float acc[16][4];
#pragma unroll
    for (int o = 0; o < 16; ++o) acc[o][0] = acc[o][1] = acc[o][2] = acc[o][3] = 0.f;
    const int64_t r_begin = int64_t(blockIdx.x) * rows_per_block;
    const int64_t r_end = r_begin + rows_per_block < M ? r_begin + rows_per_block : M;
    auto load_tile = [&](int64_t t0, int which) {
        if (t0 < r_end) {
            const int nt = int(r_end - t0 < kBwdTile ? r_end - t0 : kBwdTile);
            float* sF = wsm + which * tile_floats;
            float* sD = sF + size_t(kBwdTile) * C;
            const float* gf = feats + t0 * C;
            for (int i = threadIdx.x; i < nt * C / 4; i += blockDim.x) cp_async16(sF + 4 * i, gf + 4 * i);
            const float* gd = dB + t0 * kMaxBasis;
            for (int i = threadIdx.x; i < nt * kMaxBasis / 4; i += blockDim.x) cp_async16(sD + 4 * i, gd + 4 * i);
        }
        cp_async_commit();
    };
    load_tile(r_begin, 0);
    int buf = 0;
    for (int64_t t0 = r_begin; t0 < r_end; t0 += kBwdTile, buf ^= 1) {
        const int nt = int(r_end - t0 < kBwdTile ? r_end - t0 : kBwdTile);
        load_tile(t0 + kBwdTile, buf ^ 1);
        cp_async_wait_one();
        __syncthreads();
        const float* sF = wsm + buf * tile_floats;
        const float* sD = sF + size_t(kBwdTile) * C;
        for (int rr = rg; rr < nt; rr += kWgRowGroups) {
            const float4 f = *reinterpret_cast<const float4*>(sF + rr * C + 4 * cg);
            const float4* d = reinterpret_cast<const float4*>(sD + rr * kMaxBasis + 16 * h);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float4 dv = d[j];
                const float dd[4] = {dv.x, dv.y, dv.z, dv.w};
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    ffma2(acc[4 * j + i][0], acc[4 * j + i][1], dd[i], f.x, f.y);
                    ffma2(acc[4 * j + i][2], acc[4 * j + i][3], dd[i], f.z, f.w);
                }
            }
        }
        __syncthreads();
    }
    cp_async_wait_all();
    __syncthreads();
    // the row groups' partial sums meet in shared memory (32 x C floats)
    float* red = wsm;
    for (int i = threadIdx.x; i < kMaxBasis * C; i += blockDim.x) red[i] = 0.f;
    __syncthreads();
#pragma unroll
    for (int o = 0; o < 16; ++o)
#pragma unroll
        for (int k = 0; k < 4; ++k) atomicAdd(red + (16 * h + o) * C + 4 * cg + k, acc[o][k]);
    __syncthreads();
    for (int i = threadIdx.x; i < F * C; i += blockDim.x) atomicAdd(dWb + i, red[i]);
}

template <int FMT>
int launch_basis_tc_fmt(const CUtensorMap& ma, const CUtensorMap& mw, const CUtensorMap& mx, const CUtensorMap& mb,
                        const RenderLayout& R, const float* view, int64_t m, int stages, cudaStream_t s) {
    static bool attr_done = false;
    if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(basis_tc_kernel<FMT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(tc::kMaxSmem));
        if (e != cudaSuccess) {
            set_cuda_error(e);
            return SRF_ERR_CUDA;
        }
        attr_done = true;
    }
    const int64_t tiles = (m + 127) / 128;
    const int grid = int(tiles < num_sms() ? tiles : num_sms());
    basis_tc_kernel<FMT><<<grid, kBtThreads, bt_smem(R.C, R.k1p, stages), s>>>(
        ma, mw, mx, mb, m, R.C, R.F, view, R.lf, R.lv, R.bw, R.k1p, stages, device_flag());
    return launch_status();
}

}  // namespace

// Whether the tensor-core basis pass takes these operands: C a multiple of 4 up to
// 256, F <= 32 (B rows of 32 floats), the view block within four pieces, k1p a
// multiple of 64 and 16-byte aligned rows.
bool basis_tc_fits(const RenderLayout& R, const float* feats, const float* Wb, const float* B, const op16* x) {
    return R.C % 4 == 0 && R.C <= 256 && R.F <= 32 && R.bs == 32 && R.lv <= 4 && R.k1p % 64 == 0 && ok16(feats) &&
           ok16(Wb) && ok16(B) && ok16(x) && bt_stages(R.C, R.k1p) >= 3;
}

int launch_basis_tc(const RenderLayout& R, const float* feats, const float* Wb, const float* view, int64_t m,
                    float* B, op16* x, int fmt, cudaStream_t s) {
    if (!basis_tc_fits(R, feats, Wb, B, x)) return SRF_ERR_UNSUPPORTED;
    CUtensorMap ma, mw, mx, mb;
    if (!make_map_t(&ma, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, feats, uint64_t(R.C), uint64_t(m), uint64_t(R.C) * 4, 32,
                    128) ||
        !make_map_t(&mw, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, Wb, uint64_t(R.C), uint64_t(R.F), uint64_t(R.C) * 4, 32,
                    32) ||
        !make_map_t(&mx, CU_TENSOR_MAP_DATA_TYPE_UINT16, x, uint64_t(R.k1p), uint64_t(m), uint64_t(R.k1p) * 2, 64,
                    32) ||
        !make_map_t(&mb, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, B, uint64_t(R.bs), uint64_t(m), uint64_t(R.bs) * 4, 32, 32))
        return SRF_ERR_CUDA;
    const int stages = bt_stages(R.C, R.k1p);
    return fmt == tc::kFmtF16 ? launch_basis_tc_fmt<tc::kFmtF16>(ma, mw, mx, mb, R, view, m, stages, s)
                              : launch_basis_tc_fmt<tc::kFmtBF16>(ma, mw, mx, mb, R, view, m, stages, s);
}

// Which basis adjoint the 16-bit renderer backward runs: 1 the tensor-core pass
// where its shapes fit (default), 0 always the fused SIMT pass.
std::atomic<int> g_basis_adjoint_tc{1};

// Whether the tensor-core basis adjoint takes these operands: C a multiple of 16 up
// to 256 (the MMA's N), F <= 32, k1p a multiple of 64, 16-byte aligned rows.
bool basis_bwd_tc_fits(const RenderLayout& R, const void* dx, const float* B, const float* feats,
                       const float* d_feats, const float* dB) {
    return R.C % 16 == 0 && R.C <= 256 && R.F <= 32 && R.bs == 32 && R.k1p % 64 == 0 && ok16(dx) && ok16(B) &&
           ok16(feats) && ok16(d_feats) && ok16(dB) && bb_smem(R.C, R.k1p) <= tc::kMaxSmem;
}

int launch_basis_bwd_tc(const RenderLayout& R, const op16* dx, const float* B, const float* WbT, float* dB,
                        float* d_feats, int fmt, const float* gscale, int64_t m, cudaStream_t s) {
    CUtensorMap mdx, mb, mwt, mdb;
    if (!make_map_t(&mdx, CU_TENSOR_MAP_DATA_TYPE_UINT16, dx, uint64_t(R.k1p), uint64_t(m), uint64_t(R.k1p) * 2, 64,
                    128) ||
        !make_map_t(&mb, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, B, uint64_t(R.bs), uint64_t(m), uint64_t(R.bs) * 4, 32,
                    128) ||
        !make_map_t(&mwt, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, WbT, uint64_t(kMaxBasis), uint64_t(R.C),
                    uint64_t(kMaxBasis) * 4, 32, uint32_t(R.C)) ||
        !make_map_t(&mdb, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, dB, uint64_t(kMaxBasis), uint64_t(m),
                    uint64_t(kMaxBasis) * 4, 32, 32))
        return SRF_ERR_CUDA;
    static bool attr_done = false;
    if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(basis_bwd_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(tc::kMaxSmem));
        if (e != cudaSuccess) {
            set_cuda_error(e);
            return SRF_ERR_CUDA;
        }
        attr_done = true;
    }
    const int64_t tiles = (m + 127) / 128;
    const int grid = int(tiles < num_sms() ? tiles : num_sms());
    basis_bwd_tc_kernel<<<grid, kBbThreads, bb_smem(R.C, R.k1p), s>>>(mdx, mb, mwt, mdb, m, R.C, R.F, R.lf, R.bw,
                                                                       R.k1p, fmt, gscale, d_feats, device_flag());
    return launch_status();
}

// dWb += dB^T feats over m rows: as many resident blocks as fit, each over a
// contiguous range of rows (a multiple of the 32-row tile).
int launch_basis_wgrad(const RenderLayout& R, const float* dB, const float* feats, int64_t m, float* dWb,
                       cudaStream_t s) {
    const int threads = kWgRowGroups * (R.C / 2);   // C a multiple of 16: whole warps, at most 512
    const size_t smem = 2 * size_t(kBwdTile) * (R.C + kMaxBasis) * sizeof(float);
    if (smem > tc::kMaxSmem) return SRF_ERR_UNSUPPORTED;
    cudaError_t e = cudaFuncSetAttribute(basis_wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, basis_wgrad_kernel, threads, smem);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return SRF_ERR_CUDA;
    }
    int64_t blocks = int64_t(num_sms()) * (per_sm > 0 ? per_sm : 1);
    int64_t per = (m + blocks - 1) / blocks;
    per = (per + kBwdTile - 1) / kBwdTile * kBwdTile;
    blocks = (m + per - 1) / per;
    basis_wgrad_kernel<<<unsigned(blocks), threads, smem, s>>>(dB, feats, m, R.F, R.C, per, dWb);
    return launch_status();
}

// The basis + encoding pass: the tuner picks per (C, k1p) among the SIMT tile shapes
// (rows per thread x threads, reading the transposed basis the call writes to WbT)
// and the tensor-core pass (Wb as stored; candidate 5, where its operands fit).
// Without tuning: the first SIMT shape whose shared memory fits (128 x 2 measured
// fastest for C = 144, ahead of the tensor-core pass).
int launch_basis_encode(const RenderLayout& R, const float* feats, const float* Wb, float* WbT, const float* view,
                        int64_t m, float* B, op16* x, int fmt, cudaStream_t s) {
    if (m <= 0) return SRF_OK;
    const int C = R.C, F = R.F, k1p = R.k1p;
    auto run = [&](int i) -> int {
        if (i == 5) return launch_basis_tc(R, feats, Wb, view, m, B, x, fmt, s);
        transpose_basis_kernel<<<unsigned((C * kMaxBasis + 255) / 256), 256, 0, s>>>(Wb, F, C, WbT);
        if (const int st = launch_status()) return st;
#define SRF_ENC(RR, N)                                                                                            \
    (enc_smem_bytes(C, k1p, RR, N) <= tc::kMaxSmem                                                                \
         ? launch_basis_encode_cfg<RR, N>(feats, C, WbT, F, view, m, R.lf, R.lv, R.bw, R.bs, k1p, B, x, fmt, s)  \
         : SRF_ERR_UNSUPPORTED)
        switch (i) {
            case 0: return SRF_ENC(2, 128);
            case 1: return SRF_ENC(4, 128);
            case 2: return SRF_ENC(1, 256);
            case 3: return SRF_ENC(2, 256);
            default: return SRF_ENC(1, 128);
        }
#undef SRF_ENC
    };
    const int fallback = enc_smem_bytes(C, k1p, 2, 128) <= tc::kMaxSmem ? 0 : 4;
    const tune::Key key{tune::kSiteBasisEncode, C, k1p, 0};
    return run(tune::pick(key, 6, fallback, s, run));
}

// P = {Wb (F x C), W1 (U x k1), b1, W2 (U x U), b2, W3 (3 x U), b3}
int render_tc_forward(int C, int F, int U, int lf, int lv, int view, const float* const* P, const float* feats,
                      const float* vdirs, int64_t m, float* rgb, bool bwd, void* ws, size_t ws_bytes, int fmt,
                      srf_loss_scaler* scaler, cudaStream_t s) {
    RenderLayout R(C, F, U, lf, lv, view);
    if (!R.ok) return SRF_ERR_UNSUPPORTED;
    RenderWs w;
    if (carve_render(R, m, bwd, ws, ws_bytes, &w) > ws_bytes) return SRF_ERR_WORKSPACE;
    const TcCtx cx{fmt, scaler};
    int st;
    if ((st = pack(R.l1, P[1], w.W1, w.W1T, fmt, s))) return st;
    if ((st = pack(R.l2, P[3], w.W2, w.W2T, fmt, s))) return st;
    if (!aligned16(feats)) return SRF_ERR_ALIGN;
    if ((st = launch_basis_encode(R, feats, P[0], w.WbT, view ? vdirs : nullptr, m, w.B, w.x, fmt, s))) return st;
    if ((st = tc_linear(make_epilogue(w.h1, U, P[2], 1, fmt, cx.found_inf()), w.x, R.k1p, R.k1p, nullptr, 0, 0,
                        w.W1, R.k1p, U, 0, m, U, s)))
        return st;
    tc::GemmEpilogue ep = make_epilogue(w.h2, U, P[4], 1, fmt, cx.found_inf());
    ep.head_mode = tc::kHeadRgb;
    ep.head_w = P[5];
    ep.head_b = P[6];
    ep.head_rgb_ws = w.rgb;
    ep.head_rgb_out = rgb;
    return tc_linear(ep, w.h1, U, U, nullptr, 0, 0, w.W2, U, U, 0, m, U, s);
}

// G = gradients in P's order (accumulated); d_feats (m x C) is written.
int render_tc_backward(int C, int F, int U, int lf, int lv, int view, const float* const* P, const float* feats,
                       const float* drgb, int64_t m, float* const* G, float* d_feats, void* ws, size_t ws_bytes,
                       int fmt, srf_loss_scaler* scaler, cudaStream_t s) {
    RenderLayout R(C, F, U, lf, lv, view);
    if (!R.ok) return SRF_ERR_UNSUPPORTED;
    RenderWs w;
    if (carve_render(R, m, true, ws, ws_bytes, &w) > ws_bytes) return SRF_ERR_WORKSPACE;
    const TcCtx cx{fmt, scaler};
    int st;
    // rgb head: dZ2 (scaled), db2, dW3, db3
    if ((st = head_bwd_fused<3>(m, U, nullptr, nullptr, drgb, w.rgb, P[5], w.h2, w.dz0, nullptr, G[5], G[6], fmt,
                                cx.gscale(), cx.found_inf(), s)))
        return st;
    if ((st = wgrad_layer(R.l2, w.partial, w.partial_floats, w.dz0, w.h1, U, nullptr, 0, m, G[3], cx, s, G[4])))
        return st;
    tc::GemmEpilogue e2 = make_epilogue(w.dz1, U, nullptr, 0, fmt, cx.found_inf());
    e2.gscale = cx.gscale();
    e2.mask = w.h1;
    e2.ld_mask = U;
    if ((st = tc_linear(e2, w.dz0, U, U, nullptr, 0, 0, w.W2T, U, U, 0, m, U, s))) return st;
    if ((st = wgrad_layer(R.l1, w.partial, w.partial_floats, w.dz1, w.x, R.k1p, nullptr, 0, m, G[1], cx, s, G[2])))
        return st;
    // dX = dZ1 . W1 (k1p columns, in blocks of at most 128 output columns)
    for (int c0 = 0; c0 < R.k1p; c0 += 128) {
        const int n = R.k1p - c0 >= 128 ? 128 : 64;
        tc::GemmEpilogue e1 = make_epilogue(w.dx + c0, R.k1p, nullptr, 0, fmt, cx.found_inf());
        if ((st = tc_linear(e1, w.dz1, U, U, nullptr, 0, 0, w.W1T, U, R.k1p, c0, m, n, s))) return st;
    }
    // PE adjoint + basis layer: d_feats = dB . Wb, dWb += dB^T feats; on the tensor
    // cores (d_feats) and a SIMT reduction (dWb) where the shapes fit, else one
    // fused SIMT pass
    if (m > 0 && g_basis_adjoint_tc.load() && basis_bwd_tc_fits(R, w.dx, w.B, feats, d_feats, w.dB)) {
        transpose_basis_kernel<<<unsigned((C * kMaxBasis + 255) / 256), 256, 0, s>>>(P[0], F, C, w.WbT);
        if ((st = launch_status())) return st;
        if ((st = launch_basis_bwd_tc(R, w.dx, w.B, w.WbT, w.dB, d_feats, fmt, cx.gscale(), m, s))) return st;
        return launch_basis_wgrad(R, w.dB, feats, m, G[0], s);
    }
    const int threads = (C + 31) / 32 * 32;
    const size_t bsmem = basis_bwd_smem(C, R.bs, R.k1p);
    if (bsmem > tc::kMaxSmem) return SRF_ERR_UNSUPPORTED;
    if (bsmem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(basis_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(bsmem));
        if (e != cudaSuccess) {
            set_cuda_error(e);
            return SRF_ERR_CUDA;
        }
    }
    // as many resident blocks as registers and shared memory allow, each over a
    // contiguous range of rows
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, basis_bwd_kernel, threads, bsmem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    int64_t blocks = int64_t(num_sms()) * per_sm;
    int64_t per = (m + blocks - 1) / blocks;
    per = (per + kBwdTile - 1) / kBwdTile * kBwdTile;
    blocks = (m + per - 1) / per;
    basis_bwd_kernel<<<unsigned(blocks), threads, bsmem, s>>>(w.dx, w.B, feats, P[0], m, F, C, lf, R.bw, R.bs,
                                                             R.k1p, fmt, cx.gscale(), per, d_feats, G[0]);
    return launch_status();
}

}  // namespace srf

using namespace srf;

// ---------------------------------------------------------- raw GEMM entry --

extern "C" int srf_bf16_linear(void* out, int64_t ld_out, const void* x0, int64_t ld0, int k0, const void* x1,
                               int64_t ld1, int k1, const void* w, int64_t ldw, int w_rows, int w_row0,
                               const float* bias, int64_t m, int n, int relu, const void* mask, int64_t ld_mask,
                               float* colsum, void* stream) {
    tc::GemmEpilogue ep = make_epilogue(static_cast<op16*>(out), ld_out, bias, relu);
    ep.mask = static_cast<const op16*>(mask);
    ep.ld_mask = ld_mask;
    ep.colsum = colsum;
    return tc_linear(ep, static_cast<const op16*>(x0), ld0, k0, static_cast<const op16*>(x1), ld1, k1,
                     static_cast<const op16*>(w), ldw, w_rows, w_row0, m, n, as_stream(stream));
}

extern "C" size_t srf_bf16_wgrad_workspace_size(int n_dz, int k_total) {
    return tc_wgrad_partial_floats(n_dz, k_total) * sizeof(float);
}

extern "C" int srf_bf16_wgrad(float* partial, size_t partial_bytes, int* splits, const void* dz, int64_t ld_dz,
                              int n_dz, const void* x0, int64_t ld0, int k0, const void* x1, int64_t ld1, int k1,
                              int64_t m, void* stream) {
    if (!partial || !splits || !dz || !x0) return SRF_ERR_NULL;
    if (m <= 0) return SRF_ERR_SHAPE;
    return tc_wgrad(partial, partial_bytes / sizeof(float), static_cast<const op16*>(dz), ld_dz, n_dz,
                    static_cast<const op16*>(x0), ld0, k0, static_cast<const op16*>(x1), ld1, k1, m, splits,
                    as_stream(stream));
}

// ------------------------------------------------- TensoRF renderer entry --

static int render_fmt(int precision) {
    return precision == SRF_PRECISION_FP16 ? tc::kFmtF16 : (precision == SRF_PRECISION_BF16 ? tc::kFmtBF16 : -1);
}

extern "C" size_t srf_tensorf_renderer_workspace_size(const srf_tensorf_renderer_desc* d, int64_t m, int precision,
                                                      int for_backward) {
    if (!d || m < 0 || render_fmt(precision) < 0) return 0;
    return render_tc_workspace(d->n_comp, d->features, d->units, d->features_pe_degree, d->views_pe_degree,
                               d->view_dependent, m, for_backward != 0);
}

extern "C" int srf_tensorf_renderer_forward(const srf_tensorf_renderer_desc* d, const float* const* params,
                                            const float* feats, const float* view_dirs, int64_t m, float* rgb,
                                            int precision, int for_backward, void* workspace, size_t workspace_bytes,
                                            srf_loss_scaler* scaler, void* stream) {
    if (!d || !params || !feats || !rgb) return SRF_ERR_NULL;
    for (int i = 0; i < 7; ++i)
        if (!params[i]) return SRF_ERR_NULL;
    if (d->view_dependent && !view_dirs) return SRF_ERR_NULL;
    const int fmt = render_fmt(precision);
    if (fmt < 0) return SRF_ERR_UNSUPPORTED;
    if (m < 0) return SRF_ERR_SHAPE;
    if (m == 0) return SRF_OK;
    if (!workspace) return SRF_ERR_WORKSPACE;
    return render_tc_forward(d->n_comp, d->features, d->units, d->features_pe_degree, d->views_pe_degree,
                             d->view_dependent, params, feats, view_dirs, m, rgb, for_backward != 0, workspace,
                             workspace_bytes, fmt, scaler, as_stream(stream));
}

extern "C" int srf_nerf_mlp_fused_path(int mode) {
    if (mode > 2) return -SRF_ERR_SHAPE;   // negative: apart from the modes 0..2
    const int prev = g_mlp_fused.load();
    if (mode >= 0) g_mlp_fused.store(mode);
    return prev;
}

extern "C" int srf_tensorf_basis_adjoint_path(int tensor_cores) {
    g_basis_adjoint_tc.store(tensor_cores ? 1 : 0);
    return SRF_OK;
}

extern "C" int srf_tensorf_renderer_backward(const srf_tensorf_renderer_desc* d, const float* const* params,
                                             const float* feats, const float* d_rgb, int64_t m, float* const* grads,
                                             float* d_feats, int precision, void* workspace, size_t workspace_bytes,
                                             srf_loss_scaler* scaler, void* stream) {
    if (!d || !params || !feats || !d_rgb || !grads || !d_feats) return SRF_ERR_NULL;
    for (int i = 0; i < 7; ++i)
        if (!params[i] || !grads[i]) return SRF_ERR_NULL;
    const int fmt = render_fmt(precision);
    if (fmt < 0) return SRF_ERR_UNSUPPORTED;
    if (fmt == tc::kFmtF16 && !scaler) return SRF_ERR_NULL;
    if (m < 0) return SRF_ERR_SHAPE;
    if (m == 0) return SRF_OK;
    if (!workspace) return SRF_ERR_WORKSPACE;
    return render_tc_backward(d->n_comp, d->features, d->units, d->features_pe_degree, d->views_pe_degree,
                              d->view_dependent, params, feats, d_rgb, m, grads, d_feats, workspace, workspace_bytes,
                              fmt, scaler, as_stream(stream));
}
