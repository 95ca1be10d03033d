// BF16 tensor-core (tcgen05) path of the NeRF MLP: FP32 master weights, BF16
// activations in HBM, FP32 accumulation in tensor memory.  PE sin/cos and the
// small heads (sigma: 1 output, rgb: 3 outputs) stay in FP32 SIMT kernels.
//
// Forward per layer: one persistent tcgen05 GEMM with the bias/ReLU epilogue.
// Backward per layer: a dgrad GEMM (dZ . W^T with the ReLU mask of the forward
// activation and the bias gradient fused into its epilogue) and a split-K wgrad
// GEMM over samples (MN-major operands) reduced into the FP32 weight gradient.
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>
#include <vector>

#include "nerf_mlp.h"
#include "tc_gemm.cuh"

namespace srf {

using bf16 = __nv_bfloat16;

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

template <int BN>
int launch_gemm_bn(const CUtensorMap& a0, const CUtensorMap& a1, const CUtensorMap& b, tc::GemmShape sh,
                   tc::GemmEpilogue ep, cudaStream_t s) {
    int kb = sh.kb0 + sh.kb1;
    if (tc::SmemPlan<BN>::stages(kb) < 2) return SRF_ERR_UNSUPPORTED;
    size_t smem = tc::SmemPlan<BN>::bytes(kb);
    static bool attr_done = false;
    if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(tc::tc_gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(tc::kMaxSmem));
        if (e != cudaSuccess) {
            set_cuda_error(e);
            return SRF_ERR_CUDA;
        }
        attr_done = true;
    }
    int64_t tiles = (sh.M + tc::kBlockM - 1) / tc::kBlockM;
    int grid = int(tiles < num_sms() ? tiles : num_sms());
    tc::tc_gemm_kernel<BN><<<grid, tc::kThreads, smem, s>>>(a0, a1, b, sh, ep);
    return launch_status();
}

}  // namespace

// out[m, :n] = epilogue(x0[m, :k0] . B0^T + x1[m, :k1] . B1^T) with B the rows
// [w_row0, w_row0 + n) of the BF16 matrix w (w_rows x ldw, K-major).
int tc_linear(bf16* out, int64_t ld_out, const bf16* x0, int64_t ld0, int k0, const bf16* x1, int64_t ld1, int k1,
              const bf16* w, int64_t ldw, int w_rows, int w_row0, int64_t M, int n, const float* bias, int relu,
              const bf16* mask, int64_t ld_mask, const float* r1_row, const float* r1_col, float* colsum,
              cudaStream_t s) {
    if (M <= 0) return SRF_OK;
    if (!out || !x0 || !w) return SRF_ERR_NULL;
    if ((k0 % 64) || (k1 % 64) || k0 <= 0 || (k1 && !x1)) return SRF_ERR_SHAPE;
    if (n != 64 && n != 128 && n != 256) return SRF_ERR_UNSUPPORTED;
    if (w_row0 < 0 || w_row0 + n > w_rows || ldw < k0 + k1) return SRF_ERR_SHAPE;
    if (ld_out < n || ld0 < k0 || (x1 && ld1 < k1) || (mask && ld_mask < n)) return SRF_ERR_SHAPE;
    if (!ok16(out) || !ok16(x0) || !ok16(w) || (x1 && !ok16(x1)) || (mask && !ok16(mask))) return SRF_ERR_ALIGN;
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
    tc::GemmShape sh{M, k0 / 64, k1 / 64, w_row0};
    tc::GemmEpilogue ep{bias, relu, mask, ld_mask, r1_row, r1_col, out, ld_out, colsum, device_flag()};
    switch (n) {
        case 64: return launch_gemm_bn<64>(ma0, ma1, mb, sh, ep, s);
        case 128: return launch_gemm_bn<128>(ma0, ma1, mb, sh, ep, s);
        default: return launch_gemm_bn<256>(ma0, ma1, mb, sh, ep, s);
    }
}

// splits <= num_sms / (n_dz / 128), so splits * n_dz <= num_sms * 128
size_t tc_wgrad_partial_floats(int n_dz, int np) {
    (void)n_dz;
    return size_t(num_sms()) * 128 * np;
}

// partial[split, n, k] = sum_m dz[m, n] x[m, k] (x = [x0 | x1]); returns the split count.
int tc_wgrad(float* partial, size_t partial_floats, const bf16* dz, int64_t ld_dz, int n_dz, const bf16* x0,
             int64_t ld0, int k0, const bf16* x1, int64_t ld1, int k1, int64_t M, int* splits_out, cudaStream_t s) {
    if (n_dz % 128 || k0 % 64 || k1 % 64 || k0 <= 0 || k0 + k1 > 512) return SRF_ERR_UNSUPPORTED;
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
    if (tc::wgrad_stages(nchunks) < 2) return SRF_ERR_UNSUPPORTED;
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
    tc::WgradShape sh{M, chunk, n_dz, k0 / 64, k1 / 64};
    dim3 grid(ntile, splits);
    tc::tc_wgrad_kernel<<<grid, tc::kThreads, tc::wgrad_smem(nchunks), s>>>(mdz, m0, m1, sh, partial,
                                                                          device_flag());
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
    __host__ __device__ int kpad() const { return pad0[nsrc - 1] + padw[nsrc - 1]; }
    __host__ __device__ int kref() const { return ref0[nsrc - 1] + refw[nsrc - 1]; }
};

__device__ __forceinline__ int ref_col(const LayerMap& L, int kp) {
    for (int i = 0; i < L.nsrc; ++i) {
        int off = kp - L.pad0[i];
        if (off >= 0 && off < L.padw[i]) return off < L.refw[i] ? L.ref0[i] + off : -1;
    }
    return -1;
}

// W (n x kref, fp32) -> Wp (n x kpad, bf16) and WT (kpad x n, bf16).
__global__ void pack_weight_kernel(LayerMap L, const float* __restrict__ w, bf16* wp, bf16* wt) {
    int kp = blockIdx.x * blockDim.x + threadIdx.x;
    int n = blockIdx.y;
    int kpad = L.kpad();
    if (kp >= kpad) return;
    int rc = ref_col(L, kp);
    float v = rc >= 0 ? w[int64_t(n) * L.kref() + rc] : 0.f;
    bf16 b = __float2bfloat16_rn(v);
    wp[int64_t(n) * kpad + kp] = b;
    wt[int64_t(kp) * L.n + n] = b;
}

// grad[n, ref] += sum_s partial[s, n, kp] for the mapped columns.
__global__ void reduce_wgrad_kernel(LayerMap L, const float* __restrict__ partial, int splits, int n_dz, float* grad) {
    int kp = blockIdx.x * blockDim.x + threadIdx.x;
    int n = blockIdx.y;
    int kpad = L.kpad();
    if (kp >= kpad) return;
    int rc = ref_col(L, kp);
    if (rc < 0) return;
    float acc = 0.f;
    for (int sp = 0; sp < splits; ++sp) acc += partial[(int64_t(sp) * n_dz + n) * kpad + kp];
    grad[int64_t(n) * L.kref() + rc] += acc;
}

// enc[m] = PE(pts[m], Lp) zero-padded to enc_w; vext[m] = [PE cols pin..ppe, PE(dirs[m/div], Lv)] padded.
__global__ void encode_bf16_kernel(const float* __restrict__ pts, const float* __restrict__ dirs, int div, int64_t M,
                                   int lp, int lv, int pin, int enc_w, int vx_w, bf16* enc, bf16* vext) {
    int64_t m = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (m >= M) return;
    float p[3] = {pts[3 * m], pts[3 * m + 1], pts[3 * m + 2]};
    int ppe = 3 * (2 * lp + 1);
    bf16* e = enc + m * enc_w;
    bf16* v = vext ? vext + m * vx_w : nullptr;
    auto put = [&](int col, float val) {
        if (col < pin) e[col] = __float2bfloat16_rn(val);
        else {
            e[col] = __float2bfloat16_rn(0.f);
            if (v) v[col - pin] = __float2bfloat16_rn(val);
        }
    };
    for (int j = 0; j < 3; ++j) put(j, p[j]);
    float f = 1.f;
    for (int k = 0; k < lp; ++k) {
        for (int j = 0; j < 3; ++j) {
            float a = p[j] * f;
            put(3 * (1 + 2 * k) + j, sinf(a));
            put(3 * (2 + 2 * k) + j, cosf(a));
        }
        f *= 2.f;
    }
    for (int c = ppe; c < enc_w; ++c) e[c] = __float2bfloat16_rn(0.f);
    if (!v) return;
    int c0 = ppe - pin;
    int vpe = 0;
    if (dirs) {
        const float* d = dirs + 3 * (m / div);
        float q[3] = {d[0], d[1], d[2]};
        vpe = 3 * (2 * lv + 1);
        for (int j = 0; j < 3; ++j) v[c0 + j] = __float2bfloat16_rn(q[j]);
        float g = 1.f;
        for (int k = 0; k < lv; ++k) {
            for (int j = 0; j < 3; ++j) {
                float a = q[j] * g;
                v[c0 + 3 * (1 + 2 * k) + j] = __float2bfloat16_rn(sinf(a));
                v[c0 + 3 * (2 + 2 * k) + j] = __float2bfloat16_rn(cosf(a));
            }
            g *= 2.f;
        }
    }
    for (int c = c0 + vpe; c < vx_w; ++c) v[c] = __float2bfloat16_rn(0.f);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Heads on BF16 activations; one warp per row.  mode 0: sigma (1 output),
// 1: rgb (3), 2: sigma + rgb (4).
__global__ void head_fwd_bf16_kernel(int64_t M, int K, const bf16* __restrict__ h, const float* __restrict__ W,
                                     const float* __restrict__ b, int mode, const float* __restrict__ noise,
                                     float* sraw, float* sigma, float* rgb_ws, float* rgb_out) {
    int lane = threadIdx.x & 31;
    int64_t row = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= M) return;
    int no = mode == 0 ? 1 : (mode == 1 ? 3 : 4);
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    const bf16* hr = h + row * K;
    for (int k0 = lane * 8; k0 < K; k0 += 256) {
        uint4 raw = *reinterpret_cast<const uint4*>(hr + k0);
        uint32_t w4[4] = {raw.x, raw.y, raw.z, raw.w};
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            float2 x = tc::unpack_bf16(w4[g]);
#pragma unroll
            for (int n = 0; n < 4; ++n)
                if (n < no) d[n] += x.x * W[int64_t(n) * K + k0 + 2 * g] + x.y * W[int64_t(n) * K + k0 + 2 * g + 1];
        }
    }
#pragma unroll
    for (int n = 0; n < 4; ++n) d[n] = warp_sum(d[n]);
    if (lane != 0) return;
    int c0 = 0;
    if (mode != 1) {
        float s = d[0] + b[0];
        if (noise) s += noise[row];
        sraw[row] = s;
        sigma[row] = s > 0.f ? s : 0.f;
        c0 = 1;
    }
    if (mode != 0) {
        for (int c = 0; c < 3; ++c) {
            float v = 1.f / (1.f + expf(-(d[c0 + c] + b[c0 + c])));
            rgb_ws[3 * row + c] = v;
            rgb_out[3 * row + c] = v;
        }
    }
}

// Head adjoint: g = [dsigma*(sraw>0)] and/or [drgb * rgb * (1 - rgb)] -> dout (M x 4);
// when dz != NULL also dz[m, :] = (g . W) * (h > 0) (BF16) with its column sums.
// Threads over columns, rows looped in chunks of `rows`.
__global__ void head_bwd_bf16_kernel(int64_t M, int K, int mode, const float* __restrict__ dsigma,
                                     const float* __restrict__ drgb, const float* __restrict__ sraw,
                                     const float* __restrict__ rgb, const float* __restrict__ W,
                                     const bf16* __restrict__ h, bf16* dz, float* colsum, float* dout, float* dsig,
                                     int64_t rows) {
    int64_t r0 = int64_t(blockIdx.x) * rows;
    int64_t r1 = r0 + rows < M ? r0 + rows : M;
    float cs[2] = {0.f, 0.f};
    for (int64_t r = r0; r < r1; ++r) {
        float g[4] = {0.f, 0.f, 0.f, 0.f};
        int no = 0;
        if (mode != 1) g[no++] = sraw[r] > 0.f ? dsigma[r] : 0.f;
        if (mode != 0)
            for (int c = 0; c < 3; ++c) {
                float v = rgb[3 * r + c];
                g[no++] = drgb[3 * r + c] * v * (1.f - v);
            }
        if (threadIdx.x < 4) dout[r * 4 + threadIdx.x] = int(threadIdx.x) < no ? g[threadIdx.x] : 0.f;
        if (dsig && threadIdx.x == 0) dsig[r] = g[0];
        if (!dz) continue;
        for (int k = threadIdx.x, i = 0; k < K; k += blockDim.x, ++i) {
            float v = 0.f;
            for (int n = 0; n < no; ++n) v += g[n] * W[int64_t(n) * K + k];
            if (!(__bfloat162float(h[r * K + k]) > 0.f)) v = 0.f;
            dz[r * K + k] = __float2bfloat16_rn(v);
            cs[i & 1] += v;
        }
    }
    if (dz && colsum)
        for (int k = threadIdx.x, i = 0; k < K; k += blockDim.x, ++i) atomicAdd(colsum + k, cs[i & 1]);
}

// dW (no x K) += dout^T h ; db += colsum(dout) for heads with no <= 4 outputs.
__global__ void head_dw_bf16_kernel(int64_t M, int K, int no, const float* __restrict__ dout,
                                    const bf16* __restrict__ h, float* dw, float* db, int64_t rows) {
    int64_t r0 = int64_t(blockIdx.x) * rows;
    int64_t r1 = r0 + rows < M ? r0 + rows : M;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int64_t r = r0; r < r1; ++r) {
            float x = __bfloat162float(h[r * K + k]);
#pragma unroll
            for (int n = 0; n < 4; ++n)
                if (n < no) acc[n] += dout[r * 4 + n] * x;
        }
        for (int n = 0; n < no; ++n) atomicAdd(dw + int64_t(n) * K + k, acc[n]);
    }
    if (threadIdx.x < unsigned(no)) {
        float s = 0.f;
        for (int64_t r = r0; r < r1; ++r) s += dout[r * 4 + threadIdx.x];
        atomicAdd(db + threadIdx.x, s);
    }
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
    bf16* enc; bf16* vext;
    std::vector<bf16*> h, hv;
    bf16* feat;
    float* sraw; float* rgb;
    std::vector<bf16*> W, WT, Wv, WTv;
    bf16* Wf; bf16* WTf;
    bf16* dz0; bf16* dz1; bf16* dfeat;
    float* dsig; float* dout; float* partial; size_t partial_floats;
};

size_t carve_tc(const MlpLayout& L, const TcLayout& T, int64_t m, bool bwd, void* base, size_t cap, TcWs* out) {
    Carver c(base, cap);
    TcWs w;
    w.enc = c.take<bf16>(size_t(m) * T.enc_w);
    w.vext = L.vdep ? c.take<bf16>(size_t(m) * T.vx_w) : nullptr;
    for (int j = 0; j < L.Dp; ++j) w.h.push_back(c.take<bf16>(size_t(m) * L.Wp));
    w.feat = L.vdep ? c.take<bf16>(size_t(m) * L.Wp) : nullptr;
    for (int j = 0; L.vdep && j < L.Dv; ++j) w.hv.push_back(c.take<bf16>(size_t(m) * L.Wv));
    w.sraw = c.take<float>(size_t(m));
    w.rgb = c.take<float>(size_t(m) * 3);
    for (auto& lm : T.trunk) {
        w.W.push_back(c.take<bf16>(size_t(lm.n) * lm.kpad()));
        w.WT.push_back(c.take<bf16>(size_t(lm.n) * lm.kpad()));
    }
    w.Wf = c.take<bf16>(size_t(L.Wp) * L.Wp);
    w.WTf = c.take<bf16>(size_t(L.Wp) * L.Wp);
    for (auto& lm : T.view) {
        w.Wv.push_back(c.take<bf16>(size_t(lm.n) * lm.kpad()));
        w.WTv.push_back(c.take<bf16>(size_t(lm.n) * lm.kpad()));
    }
    int wmax = L.Wp > L.Wv ? L.Wp : L.Wv;
    if (bwd) {
        w.dz0 = c.take<bf16>(size_t(m) * wmax);
        w.dz1 = c.take<bf16>(size_t(m) * wmax);
        w.dfeat = L.vdep ? c.take<bf16>(size_t(m) * L.Wp) : nullptr;
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

int pack(const LayerMap& lm, const float* w, bf16* wp, bf16* wt, cudaStream_t s) {
    dim3 grid((lm.kpad() + 127) / 128, lm.n);
    pack_weight_kernel<<<grid, 128, 0, s>>>(lm, w, wp, wt);
    return launch_status();
}

int wgrad_layer(const LayerMap& lm, const TcWs& w, const bf16* dz, const bf16* x0, int64_t ld0, const bf16* x1,
                int64_t ld1, int64_t M, float* grad, cudaStream_t s) {
    int splits = 0;
    int st = tc_wgrad(w.partial, w.partial_floats, dz, lm.n, lm.n, x0, ld0, lm.padw[0], x1, ld1,
                      lm.nsrc > 1 ? lm.padw[1] : 0, M, &splits, s);
    if (st) return st;
    dim3 grid((lm.kpad() + 127) / 128, lm.n);
    reduce_wgrad_kernel<<<grid, 128, 0, s>>>(lm, w.partial, splits, lm.n, grad);
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
                   cudaStream_t s) {
    TcLayout T(L);
    if (!T.ok) return SRF_ERR_UNSUPPORTED;
    TcWs w;
    if (carve_tc(L, T, m, bwd, ws, ws_bytes, &w) > ws_bytes) return SRF_ERR_WORKSPACE;
    int st;
    for (int j = 0; j < L.Dp; ++j)
        if ((st = pack(T.trunk[j], P[L.idx_trunk_w(j)], w.W[j], w.WT[j], s))) return st;
    if (L.vdep) {
        if ((st = pack(T.feat, P[L.idx_feat_w()], w.Wf, w.WTf, s))) return st;
        for (int j = 0; j < L.Dv; ++j)
            if ((st = pack(T.view[j], P[L.idx_view_w(j)], w.Wv[j], w.WTv[j], s))) return st;
    }
    encode_bf16_kernel<<<grid_1d(m, 128), 128, 0, s>>>(pts, L.vpe ? dirs : nullptr, dir_div, m,
                                                       L.desc.points_pe_degree, L.desc.views_pe_degree, L.pin,
                                                       T.enc_w, T.vx_w, w.enc, w.vext);
    if ((st = launch_status())) return st;
    for (int j = 0; j < L.Dp; ++j) {
        const LayerMap& lm = T.trunk[j];
        const bf16* x0 = j == 0 || j - 1 == L.skip ? w.enc : w.h[j - 1];
        int64_t ld0 = j == 0 || j - 1 == L.skip ? T.enc_w : L.Wp;
        const bf16* x1 = lm.nsrc > 1 ? w.h[j - 1] : nullptr;
        st = tc_linear(w.h[j], L.Wp, x0, ld0, lm.padw[0], x1, L.Wp, lm.nsrc > 1 ? lm.padw[1] : 0, w.W[j], lm.kpad(),
                       lm.n, 0, m, lm.n, P[L.idx_trunk_w(j) + 1], 1, nullptr, 0, nullptr, nullptr, nullptr, s);
        if (st) return st;
    }
    const bf16* hl = w.h[L.Dp - 1];
    const int wpr = 8;
    if (!L.vdep) {
        head_fwd_bf16_kernel<<<grid_1d(m, wpr), wpr * 32, 0, s>>>(m, L.Wp, hl, P[L.idx_out_w()], P[L.idx_out_w() + 1],
                                                                  2, noise, w.sraw, sigma, w.rgb, rgb);
        return launch_status();
    }
    head_fwd_bf16_kernel<<<grid_1d(m, wpr), wpr * 32, 0, s>>>(m, L.Wp, hl, P[L.idx_out_w()], P[L.idx_out_w() + 1], 0,
                                                              noise, w.sraw, sigma, nullptr, nullptr);
    if ((st = launch_status())) return st;
    st = tc_linear(w.feat, L.Wp, hl, L.Wp, L.Wp, nullptr, 0, 0, w.Wf, L.Wp, L.Wp, 0, m, L.Wp, P[L.idx_feat_w() + 1], 0,
                   nullptr, 0, nullptr, nullptr, nullptr, s);
    if (st) return st;
    for (int j = 0; j < L.Dv; ++j) {
        const LayerMap& lm = T.view[j];
        const bf16* x0 = j == 0 ? w.feat : w.hv[j - 1];
        int64_t ld0 = j == 0 ? L.Wp : L.Wv;
        st = tc_linear(w.hv[j], L.Wv, x0, ld0, lm.padw[0], lm.nsrc > 1 ? w.vext : nullptr, T.vx_w,
                       lm.nsrc > 1 ? lm.padw[1] : 0, w.Wv[j], lm.kpad(), lm.n, 0, m, lm.n, P[L.idx_view_w(j) + 1], 1,
                       nullptr, 0, nullptr, nullptr, nullptr, s);
        if (st) return st;
    }
    head_fwd_bf16_kernel<<<grid_1d(m, wpr), wpr * 32, 0, s>>>(m, L.Wv, w.hv[L.Dv - 1], P[L.idx_rgb_w()],
                                                              P[L.idx_rgb_w() + 1], 1, nullptr, nullptr, nullptr,
                                                              w.rgb, rgb);
    return launch_status();
}

int mlp_tc_backward(const MlpLayout& L, const float* const* P, const float* dsigma, const float* drgb, int64_t m,
                    int dir_div, float* const* G, void* ws, size_t ws_bytes, cudaStream_t s) {
    (void)dir_div;
    TcLayout T(L);
    if (!T.ok) return SRF_ERR_UNSUPPORTED;
    TcWs w;
    if (carve_tc(L, T, m, true, ws, ws_bytes, &w) > ws_bytes) return SRF_ERR_WORKSPACE;
    int st;
    const int64_t rows = 512;
    const unsigned hblocks = grid_1d(m, int(rows));
    bf16* dz = w.dz0;
    bf16* dz2 = w.dz1;
    const bf16* hl = w.h[L.Dp - 1];
    if (L.vdep) {
        const bf16* hvl = w.hv[L.Dv - 1];
        head_bwd_bf16_kernel<<<hblocks, 128, 0, s>>>(m, L.Wv, 1, nullptr, drgb, nullptr, w.rgb, P[L.idx_rgb_w()], hvl,
                                                     dz, G[L.idx_view_w(L.Dv - 1) + 1], w.dout, nullptr, rows);
        if ((st = launch_status())) return st;
        head_dw_bf16_kernel<<<hblocks, 128, 0, s>>>(m, L.Wv, 3, w.dout, hvl, G[L.idx_rgb_w()], G[L.idx_rgb_w() + 1],
                                                    rows);
        if ((st = launch_status())) return st;
        for (int j = L.Dv - 1; j >= 0; --j) {
            const LayerMap& lm = T.view[j];
            const bf16* x0 = j == 0 ? w.feat : w.hv[j - 1];
            int64_t ld0 = j == 0 ? L.Wp : L.Wv;
            st = wgrad_layer(lm, w, dz, x0, ld0, lm.nsrc > 1 ? w.vext : nullptr, T.vx_w, m, G[L.idx_view_w(j)], s);
            if (st) return st;
            if (j > 0) {
                st = tc_linear(dz2, L.Wv, dz, L.Wv, L.Wv, nullptr, 0, 0, w.WTv[j], L.Wv, lm.kpad(), 0, m, L.Wv,
                               nullptr, 0, w.hv[j - 1], L.Wv, nullptr, nullptr, G[L.idx_view_w(j - 1) + 1], s);
                if (st) return st;
                std::swap(dz, dz2);
            } else {
                st = tc_linear(w.dfeat, L.Wp, dz, L.Wv, L.Wv, nullptr, 0, 0, w.WTv[0], L.Wv, lm.kpad(), 0, m, L.Wp,
                               nullptr, 0, nullptr, 0, nullptr, nullptr, G[L.idx_feat_w() + 1], s);
                if (st) return st;
            }
        }
        st = wgrad_layer(T.feat, w, w.dfeat, hl, L.Wp, nullptr, 0, m, G[L.idx_feat_w()], s);
        if (st) return st;
        // sigma head: dsig = dsigma * (sraw > 0), its weight gradient, and the
        // rank-1 term added in the feature-layer dgrad epilogue
        head_bwd_bf16_kernel<<<hblocks, 128, 0, s>>>(m, L.Wp, 0, dsigma, nullptr, w.sraw, nullptr, P[L.idx_out_w()],
                                                     hl, nullptr, nullptr, w.dout, w.dsig, rows);
        if ((st = launch_status())) return st;
        head_dw_bf16_kernel<<<hblocks, 128, 0, s>>>(m, L.Wp, 1, w.dout, hl, G[L.idx_out_w()], G[L.idx_out_w() + 1],
                                                    rows);
        if ((st = launch_status())) return st;
        st = tc_linear(dz, L.Wp, w.dfeat, L.Wp, L.Wp, nullptr, 0, 0, w.WTf, L.Wp, L.Wp, 0, m, L.Wp, nullptr, 0, hl,
                       L.Wp, w.dsig, P[L.idx_out_w()], G[L.idx_trunk_w(L.Dp - 1) + 1], s);
        if (st) return st;
    } else {
        head_bwd_bf16_kernel<<<hblocks, 128, 0, s>>>(m, L.Wp, 2, dsigma, drgb, w.sraw, w.rgb, P[L.idx_out_w()], hl, dz,
                                                     G[L.idx_trunk_w(L.Dp - 1) + 1], w.dout, nullptr, rows);
        if ((st = launch_status())) return st;
        head_dw_bf16_kernel<<<hblocks, 128, 0, s>>>(m, L.Wp, 4, w.dout, hl, G[L.idx_out_w()], G[L.idx_out_w() + 1],
                                                    rows);
        if ((st = launch_status())) return st;
    }
    for (int j = L.Dp - 1; j >= 0; --j) {
        const LayerMap& lm = T.trunk[j];
        const bf16* x0 = j == 0 || j - 1 == L.skip ? w.enc : w.h[j - 1];
        int64_t ld0 = j == 0 || j - 1 == L.skip ? T.enc_w : L.Wp;
        st = wgrad_layer(lm, w, dz, x0, ld0, lm.nsrc > 1 ? w.h[j - 1] : nullptr, L.Wp, m, G[L.idx_trunk_w(j)], s);
        if (st) return st;
        if (j == 0) break;
        int row0 = lm.nsrc > 1 ? lm.padw[0] : 0;
        st = tc_linear(dz2, L.Wp, dz, L.Wp, L.Wp, nullptr, 0, 0, w.WT[j], L.Wp, lm.kpad(), row0, m, L.Wp, nullptr, 0,
                       w.h[j - 1], L.Wp, nullptr, nullptr, G[L.idx_trunk_w(j - 1) + 1], s);
        if (st) return st;
        std::swap(dz, dz2);
    }
    return SRF_OK;
}

}  // namespace srf

using namespace srf;

// ---------------------------------------------------------- raw GEMM entry --

extern "C" int srf_bf16_linear(void* out, int64_t ld_out, const void* x0, int64_t ld0, int k0, const void* x1,
                               int64_t ld1, int k1, const void* w, int64_t ldw, int w_rows, int w_row0,
                               const float* bias, int64_t m, int n, int relu, const void* mask, int64_t ld_mask,
                               float* colsum, void* stream) {
    return tc_linear(static_cast<bf16*>(out), ld_out, static_cast<const bf16*>(x0), ld0, k0,
                     static_cast<const bf16*>(x1), ld1, k1, static_cast<const bf16*>(w), ldw, w_rows, w_row0, m, n,
                     bias, relu, static_cast<const bf16*>(mask), ld_mask, nullptr, nullptr, colsum,
                     as_stream(stream));
}

extern "C" size_t srf_bf16_wgrad_workspace_size(int n_dz, int k_total) {
    return tc_wgrad_partial_floats(n_dz, k_total) * sizeof(float);
}

extern "C" int srf_bf16_wgrad(float* partial, size_t partial_bytes, int* splits, const void* dz, int64_t ld_dz,
                              int n_dz, const void* x0, int64_t ld0, int k0, const void* x1, int64_t ld1, int k1,
                              int64_t m, void* stream) {
    if (!partial || !splits || !dz || !x0) return SRF_ERR_NULL;
    if (m <= 0) return SRF_ERR_SHAPE;
    return tc_wgrad(partial, partial_bytes / sizeof(float), static_cast<const bf16*>(dz), ld_dz, n_dz,
                    static_cast<const bf16*>(x0), ld0, k0, static_cast<const bf16*>(x1), ld1, k1, m, splits,
                    as_stream(stream));
}
