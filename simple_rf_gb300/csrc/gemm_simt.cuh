// FP32 SIMT GEMM with pluggable operand accessors and fused epilogues: the
// plain-precision path of every dense layer (the reference runs these layers as
// torch.nn.Linear in FP32).
//
// C(m,n) = sum_k A(m,k) * B(k,n); 128x128 block tile, BK = 8, 256 threads with
// 8x8 outputs each, double-buffered shared memory.  A_KC / B_KC say along which
// index the operand is contiguous in memory so that global loads coalesce.
#pragma once

#include "srf_common.cuh"

namespace srf {

// A(m, k) from up to three column segments of row-major matrices; segment s
// covers k in [kend[s-1], kend[s]) and reads row m / div[s].  An optional extra
// column (k == kend[nseg-1]) returns 1 (used to fold a bias gradient into dW).
struct SegRows {
    const float* p[3];
    int64_t ld[3];
    int kend[3];
    int div[3];
    int nseg;
    int ones_col;
    __device__ __forceinline__ float operator()(int64_t m, int k) const {
        int k0 = 0;
#pragma unroll
        for (int s = 0; s < 3; ++s) {
            if (s < nseg && k < kend[s]) {
                int64_t row = div[s] == 1 ? m : m / div[s];
                return p[s][row * ld[s] + (k - k0)];
            }
            if (s < nseg) k0 = kend[s];
        }
        return ones_col ? 1.f : 0.f;
    }
};

// (i, j) -> p[i * ld + j + col0]
struct RowMajor {
    const float* p;
    int64_t ld;
    int col0;
    __device__ __forceinline__ float operator()(int64_t i, int j) const { return p[i * ld + j + col0]; }
};

// (i, j) -> p[j * ld + i + col0]   (the transpose of RowMajor)
struct ColMajor {
    const float* p;
    int64_t ld;
    int col0;
    __device__ __forceinline__ float operator()(int64_t i, int j) const { return p[int64_t(j) * ld + i + col0]; }
};

// B(k, n) = W[n, col0 + k] for a torch Linear weight (out, in): contiguous in k.
struct WeightT {
    const float* w;
    int64_t ld;
    int col0;
    __device__ __forceinline__ float operator()(int64_t k, int n) const { return w[int64_t(n) * ld + col0 + k]; }
};

template <bool A_KC, bool B_KC, class AOp, class BOp, class Epi>
__global__ void __launch_bounds__(256) sgemm_kernel(int64_t M, int N, int64_t K, int64_t kchunk,
                                                    const int* m_dev, int m_dev_is_k, AOp A, BOp B, Epi epi) {
    __shared__ __align__(16) float As[2][8][132];
    __shared__ __align__(16) float Bs[2][8][132];
    if (m_dev) {
        int64_t dyn = *m_dev;
        if (m_dev_is_k) {
            if (dyn < K) K = dyn;
        } else if (dyn < M) {
            M = dyn;
        }
    }
    const int tid = threadIdx.x;
    const int64_t m0 = int64_t(blockIdx.x) * 128;
    const int n0 = blockIdx.y * 128;
    if (m0 >= M) return;
    const int64_t kbeg = int64_t(blockIdx.z) * kchunk;
    if (kbeg >= K) return;
    const int64_t kend = kbeg + kchunk < K ? kbeg + kchunk : K;

    float ra[4], rb[4];
    auto loadA = [&](int64_t k0) {
        if (A_KC) {
            int row = tid >> 1, kk = (tid & 1) * 4;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                int64_t k = k0 + kk + q;
                ra[q] = (m0 + row < M && k < kend) ? A(m0 + row, int(k)) : 0.f;
            }
        } else {
            int kk = tid >> 5, row = (tid & 31) * 4;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                int64_t k = k0 + kk;
                ra[q] = (m0 + row + q < M && k < kend) ? A(m0 + row + q, int(k)) : 0.f;
            }
        }
    };
    auto storeA = [&](int buf) {
        if (A_KC) {
            int row = tid >> 1, kk = (tid & 1) * 4;
#pragma unroll
            for (int q = 0; q < 4; ++q) As[buf][kk + q][row] = ra[q];
        } else {
            int kk = tid >> 5, row = (tid & 31) * 4;
#pragma unroll
            for (int q = 0; q < 4; ++q) As[buf][kk][row + q] = ra[q];
        }
    };
    auto loadB = [&](int64_t k0) {
        if (B_KC) {
            int col = tid >> 1, kk = (tid & 1) * 4;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                int64_t k = k0 + kk + q;
                rb[q] = (n0 + col < N && k < kend) ? B(k, n0 + col) : 0.f;
            }
        } else {
            int kk = tid >> 5, col = (tid & 31) * 4;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                int64_t k = k0 + kk;
                rb[q] = (n0 + col + q < N && k < kend) ? B(k, n0 + col + q) : 0.f;
            }
        }
    };
    auto storeB = [&](int buf) {
        if (B_KC) {
            int col = tid >> 1, kk = (tid & 1) * 4;
#pragma unroll
            for (int q = 0; q < 4; ++q) Bs[buf][kk + q][col] = rb[q];
        } else {
            int kk = tid >> 5, col = (tid & 31) * 4;
#pragma unroll
            for (int q = 0; q < 4; ++q) Bs[buf][kk][col + q] = rb[q];
        }
    };

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

    const int tx = tid & 15, ty = tid >> 4;
    loadA(kbeg);
    loadB(kbeg);
    storeA(0);
    storeB(0);
    __syncthreads();
    int buf = 0;
    for (int64_t k0 = kbeg; k0 < kend; k0 += 8) {
        bool more = k0 + 8 < kend;
        if (more) {
            loadA(k0 + 8);
            loadB(k0 + 8);
        }
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
            float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4]);
            float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][64 + ty * 4]);
            float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
            float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][64 + tx * 4]);
            float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] += av[i] * bv[j];
        }
        if (more) {
            storeA(buf ^ 1);
            storeB(buf ^ 1);
        }
        __syncthreads();
        buf ^= 1;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        int64_t m = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            int n = n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + j - 4);
            if (n < N) epi(m, n, acc[i][j]);
        }
    }
}

// ---------------------------------------------------------------- epilogues --

struct EpiStore {   // y = act(acc + bias)
    float* y;
    int64_t ldy;
    const float* bias;
    int act;
    __device__ __forceinline__ void operator()(int64_t m, int n, float v) const {
        if (bias) v += bias[n];
        if (act == SRF_ACT_RELU) v = relu_f(v);
        else if (act == SRF_ACT_SIGMOID) v = sigmoid_f(v);
        y[m * ldy + n] = v;
    }
};

struct EpiMasked {  // dx = acc * (mask > 0)  (ReLU derivative taken from the forward output)
    float* y;
    int64_t ldy;
    const float* mask;
    int64_t ldm;
    int accumulate;
    __device__ __forceinline__ void operator()(int64_t m, int n, float v) const {
        if (mask && !(mask[m * ldm + n] > 0.f)) v = 0.f;
        if (accumulate) y[m * ldy + n] += v;
        else y[m * ldy + n] = v;
    }
};

struct EpiAtomicW {  // split-K weight gradient; column k_in is the bias gradient
    float* dw;
    int64_t ldw;
    float* db;
    int k_in;
    __device__ __forceinline__ void operator()(int64_t m, int n, float v) const {
        if (n < k_in) atomicAdd(dw + m * ldw + n, v);
        else if (db) atomicAdd(db + m, v);
    }
};

template <bool A_KC, bool B_KC, class AOp, class BOp, class Epi>
inline int sgemm(cudaStream_t s, int64_t M, int N, int64_t K, int splits, const int* m_dev, int m_dev_is_k,
                 AOp a, BOp b, Epi e) {
    if (M <= 0 || N <= 0 || K <= 0) return SRF_OK;
    if (splits < 1) splits = 1;
    int64_t kchunk = (K + splits - 1) / splits;
    kchunk = (kchunk + 7) / 8 * 8;
    int64_t z = (K + kchunk - 1) / kchunk;
    dim3 grid(unsigned((M + 127) / 128), unsigned((N + 127) / 128), unsigned(z));
    sgemm_kernel<A_KC, B_KC><<<grid, 256, 0, s>>>(M, N, K, kchunk, m_dev, m_dev_is_k, a, b, e);
    return launch_status();
}

}  // namespace srf
