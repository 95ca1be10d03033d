// NeRF MLP (SimpleNeRF17.py:616-785) forward and backward, and the generic
// dense layer used by the TensoRF renderer.  This file holds the FP32 plain
// path (SIMT GEMMs with fused bias/ReLU/mask epilogues) and the host-side
// orchestration shared with the BF16 tensor-core path (nerf_mlp_tc.cu).
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gemm_simt.cuh"
#include "nerf_mlp.h"

namespace srf {
namespace {

// ------------------------------------------------------------ head kernels --
// Heads with at most four outputs run one warp per row (lanes stride over K)
// instead of wasting a 128-wide GEMM tile.
enum HeadMode { kHeadSigma = 0, kHeadRgb = 1, kHeadSigmaRgb = 2 };

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void head_fwd_kernel(int64_t M, int K, const float* __restrict__ h, int64_t ldh,
                                const float* __restrict__ W, const float* __restrict__ b, int mode,
                                const float* __restrict__ noise, float* sraw, float* sigma, float* rgb_ws,
                                float* rgb_out) {
    int lane = threadIdx.x & 31;
    int64_t row = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= M) return;
    int no = mode == kHeadSigma ? 1 : (mode == kHeadRgb ? 3 : 4);
    float d[4] = {0.f, 0.f, 0.f, 0.f};
    const float* hr = h + row * ldh;
    for (int k = lane; k < K; k += 32) {
        float x = hr[k];
#pragma unroll
        for (int n = 0; n < 4; ++n)
            if (n < no) d[n] += x * W[int64_t(n) * K + k];
    }
#pragma unroll
    for (int n = 0; n < 4; ++n) d[n] = warp_sum(d[n]);
    if (lane != 0) return;
    int c0 = 0;
    if (mode != kHeadRgb) {
        float s = d[0] + b[0];
        if (noise) s = s + noise[row];
        sraw[row] = s;
        sigma[row] = relu_f(s);
        c0 = 1;
    }
    if (mode != kHeadSigma) {
        for (int c = 0; c < 3; ++c) {
            float v = sigmoid_f(d[c0 + c] + b[c0 + c]);
            rgb_ws[3 * row + c] = v;
            if (rgb_out) rgb_out[3 * row + c] = v;
        }
    }
}

// dOut (M x 4, ld 4) from the output gradients, and dZ = (dH_in + dOut . W) * (h > 0).
__global__ void head_bwd_kernel(int64_t M, int K, int mode, const float* __restrict__ dsigma,
                                const float* __restrict__ drgb, const float* __restrict__ sraw,
                                const float* __restrict__ rgb, const float* __restrict__ W, const float* dh_in,
                                int64_t ld_in, const float* __restrict__ hmask, int64_t ldm, float* dz,
                                int64_t ldz, float* dout) {
    int lane = threadIdx.x & 31;
    int64_t row = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= M) return;
    float g[4] = {0.f, 0.f, 0.f, 0.f};
    int no = 0;
    if (mode != kHeadRgb) g[no++] = sraw[row] > 0.f ? dsigma[row] : 0.f;
    if (mode != kHeadSigma) {
        for (int c = 0; c < 3; ++c) {
            float r = rgb[3 * row + c];
            g[no++] = drgb[3 * row + c] * r * (1.f - r);
        }
    }
    if (lane < 4) dout[row * 4 + lane] = lane < no ? g[lane] : 0.f;
    for (int k = lane; k < K; k += 32) {
        float v = dh_in ? dh_in[row * ld_in + k] : 0.f;
#pragma unroll
        for (int n = 0; n < 4; ++n)
            if (n < no) v += g[n] * W[int64_t(n) * K + k];
        if (!(hmask[row * ldm + k] > 0.f)) v = 0.f;
        dz[row * ldz + k] = v;
    }
}

// dW (no x K) += dOut^T h ; db += colsum(dOut), for no <= 4 outputs.
__global__ void small_dw_kernel(int64_t M, int K, int no, const float* __restrict__ dout,
                                const float* __restrict__ h, int64_t ldh, float* dw, float* db, int64_t rows) {
    int64_t r0 = int64_t(blockIdx.x) * rows;
    int64_t r1 = r0 + rows < M ? r0 + rows : M;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int64_t r = r0; r < r1; ++r) {
            float x = h[r * ldh + k];
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

__global__ void pe_rows_kernel(float* out, int64_t ld, const float* __restrict__ x, int64_t m, int dims,
                               int degree, const int* m_dev) {
    int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (m_dev && *m_dev < m) m = *m_dev;
    if (idx >= m * dims) return;
    int64_t row = idx / dims;
    int j = int(idx % dims);
    float v = x[row * dims + j];
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

__global__ void pe_bwd_kernel(float* dx, const float* __restrict__ x, const float* __restrict__ dout, int64_t ld,
                              int64_t m, const int* m_dev, int dims, int degree) {
    int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (m_dev && *m_dev < m) m = *m_dev;
    if (idx >= m * dims) return;
    int64_t row = idx / dims;
    int j = int(idx % dims);
    float v = x[row * dims + j];
    const float* g = dout + row * ld;
    float acc = g[j];
    float f = 1.f;
    for (int k = 0; k < degree; ++k) {
        float a = v * f;
        acc += f * (g[dims * (1 + 2 * k) + j] * cosf(a) - g[dims * (2 + 2 * k) + j] * sinf(a));
        f *= 2.f;
    }
    dx[row * dims + j] = acc;
}

__global__ void act_grad_kernel(float* dz, int64_t ldz, const float* dy, int64_t lddy, const float* y, int64_t ldy,
                                int64_t m, const int* m_dev, int n, int act) {
    int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (m_dev && *m_dev < m) m = *m_dev;
    if (idx >= m * n) return;
    int64_t r = idx / n;
    int c = int(idx % n);
    float g = dy[r * lddy + c];
    float v = act != SRF_ACT_NONE ? y[r * ldy + c] : 0.f;
    if (act == SRF_ACT_RELU) g = v > 0.f ? g : 0.f;
    else if (act == SRF_ACT_SIGMOID) g = g * v * (1.f - v);
    dz[r * ldz + c] = g;
}

int dw_splits(int64_t M_out, int N_in, int64_t K_rows) {
    int64_t tiles = ((M_out + 127) / 128) * ((N_in + 127) / 128);
    int64_t want = (2 * 152 + tiles - 1) / tiles;
    int64_t cap = (K_rows + 2047) / 2048;
    if (want > cap) want = cap;
    if (want < 1) want = 1;
    if (want > 4096) want = 4096;
    return int(want);
}

SegRows seg1(const float* p, int64_t ld, int k) {
    SegRows s{};
    s.p[0] = p; s.ld[0] = ld; s.kend[0] = k; s.div[0] = 1; s.nseg = 1; s.ones_col = 0;
    return s;
}

}  // namespace

// ------------------------------------------------------------ layout --------

MlpLayout::MlpLayout(const srf_nerf_mlp_desc& d) : desc(d) {
    Dp = d.points_net_depth; Wp = d.points_net_width; Dv = d.views_net_depth; Wv = d.views_net_width;
    ppe = 3 * (2 * d.points_pe_degree + 1);
    pin = d.points_sigma_pe_degree >= 0 ? 3 * (2 * d.points_sigma_pe_degree + 1) : ppe;
    vpe = d.use_view_dirs ? 3 * (2 * d.views_pe_degree + 1) : 0;
    vin = vpe + (ppe - pin);
    vdep = d.view_dependent_rgb != 0;
    skip = d.skip_layer;
    valid = Dp >= 1 && Wp >= 1 && ppe >= 3 && pin <= ppe && (!vdep || (d.use_view_dirs && Dv >= 1 && Wv >= 1)) &&
            skip < Dp - 1 && d.points_pe_degree <= 24 && d.views_pe_degree <= 24 && Wp <= 4096 && Wv <= 4096;
    auto add = [&](const std::string& n, int rows, int cols) {
        names.push_back(n);
        shapes.push_back({rows, cols});
    };
    for (int j = 0; j < Dp; ++j) {
        int kin = j == 0 ? pin : (j - 1 == skip ? Wp + pin : Wp);
        layer_k.push_back(kin);
        add("pts_linears." + std::to_string(j) + ".weight", Wp, kin);
        add("pts_linears." + std::to_string(j) + ".bias", Wp, 0);
    }
    if (vdep) {
        for (int j = 0; j < Dv; ++j) {
            int kin = j == 0 ? vin + Wp : Wv;
            view_k.push_back(kin);
            add("views_linears." + std::to_string(j) + ".weight", Wv, kin);
            add("views_linears." + std::to_string(j) + ".bias", Wv, 0);
        }
    }
    add("pts_output_linear.weight", vdep ? 1 : 4, Wp);
    add("pts_output_linear.bias", vdep ? 1 : 4, 0);
    if (vdep) {
        add("feature_linear.weight", Wp, Wp);
        add("feature_linear.bias", Wp, 0);
        add("views_output_linear.weight", 3, Wv);
        add("views_output_linear.bias", 3, 0);
    }
}

int MlpLayout::idx_trunk_w(int j) const { return 2 * j; }
int MlpLayout::idx_view_w(int j) const { return 2 * Dp + 2 * j; }
int MlpLayout::idx_out_w() const { return 2 * Dp + (vdep ? 2 * Dv : 0); }
int MlpLayout::idx_feat_w() const { return idx_out_w() + 2; }
int MlpLayout::idx_rgb_w() const { return idx_out_w() + 4; }

SegRows MlpLayout::trunk_input(int j, const float* enc, float* const* h) const {
    if (j == 0) return seg1(enc, ppe, pin);
    if (j - 1 == skip) {
        SegRows s{};
        s.p[0] = enc; s.ld[0] = ppe; s.kend[0] = pin; s.div[0] = 1;
        s.p[1] = h[j - 1]; s.ld[1] = Wp; s.kend[1] = pin + Wp; s.div[1] = 1;
        s.nseg = 2;
        s.ones_col = 0;
        return s;
    }
    return seg1(h[j - 1], Wp, Wp);
}

SegRows MlpLayout::view_input(int j, const float* feat, const float* enc, const float* encv, int dir_div,
                              float* const* hv) const {
    if (j > 0) return seg1(hv[j - 1], Wv, Wv);
    SegRows s{};
    int n = 0, k = 0;
    s.p[n] = feat; s.ld[n] = Wp; k += Wp; s.kend[n] = k; s.div[n] = 1; ++n;
    if (ppe > pin) { s.p[n] = enc + pin; s.ld[n] = ppe; k += ppe - pin; s.kend[n] = k; s.div[n] = 1; ++n; }
    if (vpe > 0) { s.p[n] = encv; s.ld[n] = vpe; k += vpe; s.kend[n] = k; s.div[n] = dir_div; ++n; }
    s.nseg = n;
    s.ones_col = 0;
    return s;
}

// FP32 workspace layout.
struct F32Ws {
    float* enc; float* encv; std::vector<float*> h; float* feat; std::vector<float*> hv;
    float* sraw; float* rgb; float* dout; float* dA; float* dB; float* dfeat;
};

// The per-ray view encoding is sized for one ray per sample so that the layout
// does not depend on dir_div.
static size_t carve_f32(const MlpLayout& L, int64_t m, bool bwd, void* base, size_t cap, F32Ws* w) {
    Carver c(base, cap);
    F32Ws t;
    t.enc = c.take<float>(size_t(m) * L.ppe);
    t.encv = c.take<float>(size_t(m) * (L.vpe ? L.vpe : 1));
    int nh = bwd ? L.Dp : 2;
    for (int i = 0; i < nh; ++i) t.h.push_back(c.take<float>(size_t(m) * L.Wp));
    t.feat = L.vdep ? c.take<float>(size_t(m) * L.Wp) : nullptr;
    int nv = L.vdep ? (bwd ? L.Dv : 2) : 0;
    for (int i = 0; i < nv; ++i) t.hv.push_back(c.take<float>(size_t(m) * L.Wv));
    t.sraw = c.take<float>(size_t(m));
    t.rgb = c.take<float>(size_t(m) * 3);
    if (bwd) {
        int wmax = L.Wp > L.Wv ? L.Wp : L.Wv;
        t.dout = c.take<float>(size_t(m) * 4);
        t.dA = c.take<float>(size_t(m) * wmax);
        t.dB = c.take<float>(size_t(m) * wmax);
        t.dfeat = c.take<float>(size_t(m) * L.Wp);
    } else {
        t.dout = t.dA = t.dB = t.dfeat = nullptr;
    }
    if (w) *w = t;
    return c.used;
}

size_t mlp_f32_workspace(const MlpLayout& L, int64_t m, bool bwd) {
    return carve_f32(L, m, bwd, nullptr, ~size_t(0), nullptr);
}

int mlp_f32_forward(const MlpLayout& L, const float* const* P, const float* pts, const float* dirs, int dir_div,
                    int64_t m, const float* noise, float* sigma, float* rgb, bool bwd, void* ws, size_t ws_bytes,
                    cudaStream_t s) {
    int64_t rays = (m + dir_div - 1) / dir_div;
    F32Ws w;
    size_t need = carve_f32(L, m, bwd, ws, ws_bytes, &w);
    if (need > ws_bytes) return SRF_ERR_WORKSPACE;
    int st;
    pe_rows_kernel<<<grid_1d(m * 3, 256), 256, 0, s>>>(w.enc, L.ppe, pts, m, 3, L.desc.points_pe_degree, nullptr);
    if ((st = launch_status())) return st;
    if (L.vpe) {
        pe_rows_kernel<<<grid_1d(rays * 3, 256), 256, 0, s>>>(w.encv, L.vpe, dirs, rays, 3, L.desc.views_pe_degree,
                                                              nullptr);
        if ((st = launch_status())) return st;
    }
    std::vector<float*> hbuf(L.Dp);
    for (int j = 0; j < L.Dp; ++j) hbuf[j] = bwd ? w.h[j] : w.h[j & 1];
    for (int j = 0; j < L.Dp; ++j) {
        SegRows a = L.trunk_input(j, w.enc, hbuf.data());
        st = sgemm<true, true>(s, m, L.Wp, L.layer_k[j], 1, nullptr, 0, a,
                               WeightT{P[L.idx_trunk_w(j)], L.layer_k[j], 0},
                               EpiStore{hbuf[j], L.Wp, P[L.idx_trunk_w(j) + 1], SRF_ACT_RELU});
        if (st) return st;
    }
    const float* hl = hbuf[L.Dp - 1];
    const int wpr = 8;
    if (!L.vdep) {
        head_fwd_kernel<<<grid_1d(m, wpr), wpr * 32, 0, s>>>(m, L.Wp, hl, L.Wp, P[L.idx_out_w()], P[L.idx_out_w() + 1],
                                                             kHeadSigmaRgb, noise, w.sraw, sigma, w.rgb, rgb);
        return launch_status();
    }
    head_fwd_kernel<<<grid_1d(m, wpr), wpr * 32, 0, s>>>(m, L.Wp, hl, L.Wp, P[L.idx_out_w()], P[L.idx_out_w() + 1],
                                                         kHeadSigma, noise, w.sraw, sigma, nullptr, nullptr);
    if ((st = launch_status())) return st;
    st = sgemm<true, true>(s, m, L.Wp, L.Wp, 1, nullptr, 0, seg1(hl, L.Wp, L.Wp),
                           WeightT{P[L.idx_feat_w()], L.Wp, 0}, EpiStore{w.feat, L.Wp, P[L.idx_feat_w() + 1],
                                                                        SRF_ACT_NONE});
    if (st) return st;
    std::vector<float*> vbuf(L.Dv);
    for (int j = 0; j < L.Dv; ++j) vbuf[j] = bwd ? w.hv[j] : w.hv[j & 1];
    for (int j = 0; j < L.Dv; ++j) {
        SegRows a = L.view_input(j, w.feat, w.enc, w.encv, dir_div, vbuf.data());
        st = sgemm<true, true>(s, m, L.Wv, L.view_k[j], 1, nullptr, 0, a, WeightT{P[L.idx_view_w(j)], L.view_k[j], 0},
                               EpiStore{vbuf[j], L.Wv, P[L.idx_view_w(j) + 1], SRF_ACT_RELU});
        if (st) return st;
    }
    head_fwd_kernel<<<grid_1d(m, wpr), wpr * 32, 0, s>>>(m, L.Wv, vbuf[L.Dv - 1], L.Wv, P[L.idx_rgb_w()],
                                                         P[L.idx_rgb_w() + 1], kHeadRgb, nullptr, nullptr, nullptr,
                                                         w.rgb, rgb);
    return launch_status();
}

// Weight gradient dW (+)= dZ^T A (split over rows), bias gradient via the ones column.
static int weight_grad(cudaStream_t s, int64_t m, const float* dz, int n_out, SegRows a, int k_in, float* dw,
                       float* db, const int* m_dev) {
    a.ones_col = 1;
    return sgemm<false, false>(s, n_out, k_in + 1, m, dw_splits(n_out, k_in + 1, m), m_dev, 1,
                               ColMajor{dz, n_out, 0}, a, EpiAtomicW{dw, k_in, db, k_in});
}

int mlp_f32_backward(const MlpLayout& L, const float* const* P, const float* dsigma, const float* drgb, int64_t m,
                     int dir_div, float* const* G, void* ws, size_t ws_bytes, cudaStream_t s) {
    F32Ws w;
    size_t need = carve_f32(L, m, true, ws, ws_bytes, &w);
    if (need > ws_bytes) return SRF_ERR_WORKSPACE;
    int st;
    const int wpr = 8;
    float* hl = w.h[L.Dp - 1];
    float* dz = w.dA;      // gradient w.r.t. the current layer's pre-activation
    float* dz2 = w.dB;
    if (L.vdep) {
        float* hvl = w.hv[L.Dv - 1];
        head_bwd_kernel<<<grid_1d(m, wpr), wpr * 32, 0, s>>>(m, L.Wv, kHeadRgb, nullptr, drgb, nullptr, w.rgb,
                                                             P[L.idx_rgb_w()], nullptr, 0, hvl, L.Wv, dz, L.Wv,
                                                             w.dout);
        if ((st = launch_status())) return st;
        small_dw_kernel<<<grid_1d(m, 1024), 256, 0, s>>>(m, L.Wv, 3, w.dout, hvl, L.Wv, G[L.idx_rgb_w()],
                                                         G[L.idx_rgb_w() + 1], 1024);
        if ((st = launch_status())) return st;
        for (int j = L.Dv - 1; j >= 0; --j) {
            SegRows a = L.view_input(j, w.feat, w.enc, w.encv, dir_div, w.hv.data());
            st = weight_grad(s, m, dz, L.Wv, a, L.view_k[j], G[L.idx_view_w(j)], G[L.idx_view_w(j) + 1], nullptr);
            if (st) return st;
            if (j > 0) {
                st = sgemm<true, false>(s, m, L.Wv, L.Wv, 1, nullptr, 0, RowMajor{dz, L.Wv, 0},
                                        RowMajor{P[L.idx_view_w(j)], L.view_k[j], 0},
                                        EpiMasked{dz2, L.Wv, w.hv[j - 1], L.Wv, 0});
            } else {
                st = sgemm<true, false>(s, m, L.Wp, L.Wv, 1, nullptr, 0, RowMajor{dz, L.Wv, 0},
                                        RowMajor{P[L.idx_view_w(0)], L.view_k[0], 0},
                                        EpiMasked{w.dfeat, L.Wp, nullptr, 0, 0});
            }
            if (st) return st;
            std::swap(dz, dz2);
        }
        // feature_linear: dW_f, then dH_last = dfeat . W_f
        st = weight_grad(s, m, w.dfeat, L.Wp, seg1(hl, L.Wp, L.Wp), L.Wp, G[L.idx_feat_w()], G[L.idx_feat_w() + 1],
                         nullptr);
        if (st) return st;
        st = sgemm<true, false>(s, m, L.Wp, L.Wp, 1, nullptr, 0, RowMajor{w.dfeat, L.Wp, 0},
                                RowMajor{P[L.idx_feat_w()], L.Wp, 0}, EpiMasked{dz2, L.Wp, nullptr, 0, 0});
        if (st) return st;
        // sigma head: dZ_last = (dH_last + dsig' W_sigma) * (h_last > 0)
        head_bwd_kernel<<<grid_1d(m, wpr), wpr * 32, 0, s>>>(m, L.Wp, kHeadSigma, dsigma, nullptr, w.sraw, nullptr,
                                                             P[L.idx_out_w()], dz2, L.Wp, hl, L.Wp, dz, L.Wp, w.dout);
        if ((st = launch_status())) return st;
        small_dw_kernel<<<grid_1d(m, 1024), 256, 0, s>>>(m, L.Wp, 1, w.dout, hl, L.Wp, G[L.idx_out_w()],
                                                         G[L.idx_out_w() + 1], 1024);
        if ((st = launch_status())) return st;
    } else {
        head_bwd_kernel<<<grid_1d(m, wpr), wpr * 32, 0, s>>>(m, L.Wp, kHeadSigmaRgb, dsigma, drgb, w.sraw, w.rgb,
                                                             P[L.idx_out_w()], nullptr, 0, hl, L.Wp, dz, L.Wp, w.dout);
        if ((st = launch_status())) return st;
        small_dw_kernel<<<grid_1d(m, 1024), 256, 0, s>>>(m, L.Wp, 4, w.dout, hl, L.Wp, G[L.idx_out_w()],
                                                         G[L.idx_out_w() + 1], 1024);
        if ((st = launch_status())) return st;
    }
    for (int j = L.Dp - 1; j >= 0; --j) {
        SegRows a = L.trunk_input(j, w.enc, w.h.data());
        st = weight_grad(s, m, dz, L.Wp, a, L.layer_k[j], G[L.idx_trunk_w(j)], G[L.idx_trunk_w(j) + 1], nullptr);
        if (st) return st;
        if (j == 0) break;
        int col0 = (j - 1 == L.skip) ? L.pin : 0;
        st = sgemm<true, false>(s, m, L.Wp, L.Wp, 1, nullptr, 0, RowMajor{dz, L.Wp, 0},
                                RowMajor{P[L.idx_trunk_w(j)], L.layer_k[j], col0},
                                EpiMasked{dz2, L.Wp, w.h[j - 1], L.Wp, 0});
        if (st) return st;
        std::swap(dz, dz2);
    }
    return SRF_OK;
}

}  // namespace srf

using namespace srf;

// ------------------------------------------------------------ C ABI ---------

extern "C" int srf_nerf_mlp_num_params(const srf_nerf_mlp_desc* desc) {
    if (!desc) return -SRF_ERR_NULL;
    MlpLayout L(*desc);
    return int(L.names.size());
}

extern "C" int srf_nerf_mlp_param_info(const srf_nerf_mlp_desc* desc, int index, char* name, int name_len,
                                       int64_t* numel) {
    if (!desc) return SRF_ERR_NULL;
    MlpLayout L(*desc);
    if (index < 0 || index >= int(L.names.size())) return SRF_ERR_SHAPE;
    if (name && name_len > 0) {
        std::strncpy(name, L.names[index].c_str(), size_t(name_len) - 1);
        name[name_len - 1] = 0;
    }
    if (numel) {
        auto sh = L.shapes[index];
        *numel = int64_t(sh.first) * (sh.second ? sh.second : 1);
    }
    return SRF_OK;
}

extern "C" size_t srf_nerf_mlp_workspace_size(const srf_nerf_mlp_desc* desc, int64_t m, int precision,
                                              int for_backward) {
    if (!desc || m < 0) return 0;
    MlpLayout L(*desc);
    if (!L.valid) return 0;
    if (precision == SRF_PRECISION_BF16 || precision == SRF_PRECISION_FP16)
        return mlp_tc_workspace(L, m, for_backward != 0);
    if (precision != SRF_PRECISION_FP32) return 0;
    return mlp_f32_workspace(L, m, for_backward != 0);
}

static int check_params(const MlpLayout& L, const float* const* p) {
    if (!p) return SRF_ERR_NULL;
    for (size_t i = 0; i < L.names.size(); ++i)
        if (!p[i]) return SRF_ERR_NULL;
    return SRF_OK;
}

extern "C" int srf_nerf_mlp_forward(const srf_nerf_mlp_desc* desc, const float* const* params, const float* pts,
                                    const float* dirs, int dir_div, int64_t m, const float* sigma_noise,
                                    float* sigma, float* rgb, int precision, int for_backward, void* workspace,
                                    size_t workspace_bytes, srf_loss_scaler* scaler, void* stream) {
    if (!desc || !pts || !sigma || !rgb) return SRF_ERR_NULL;
    MlpLayout L(*desc);
    if (!L.valid) return SRF_ERR_UNSUPPORTED;
    if (m < 0 || dir_div < 1) return SRF_ERR_SHAPE;
    if (L.vpe && !dirs) return SRF_ERR_NULL;
    int st = check_params(L, params);
    if (st) return st;
    if (m == 0) return SRF_OK;
    if (!workspace) return SRF_ERR_WORKSPACE;
    if (precision == SRF_PRECISION_BF16 || precision == SRF_PRECISION_FP16)
        return mlp_tc_forward(L, params, pts, dirs, dir_div, m, sigma_noise, sigma, rgb, for_backward != 0, workspace,
                              workspace_bytes, precision == SRF_PRECISION_FP16 ? 1 : 0, scaler, as_stream(stream));
    if (precision != SRF_PRECISION_FP32) return SRF_ERR_UNSUPPORTED;
    return mlp_f32_forward(L, params, pts, dirs, dir_div, m, sigma_noise, sigma, rgb, for_backward != 0, workspace,
                           workspace_bytes, as_stream(stream));
}

extern "C" int srf_nerf_mlp_backward(const srf_nerf_mlp_desc* desc, const float* const* params, const float* dsigma,
                                     const float* drgb, int dir_div, int64_t m, float* const* grads, int accumulate,
                                     int precision, void* workspace, size_t workspace_bytes, srf_loss_scaler* scaler,
                                     void* stream) {
    if (!desc || !dsigma || !drgb || !grads) return SRF_ERR_NULL;
    if (precision == SRF_PRECISION_FP16 && !scaler) return SRF_ERR_NULL;
    MlpLayout L(*desc);
    if (!L.valid) return SRF_ERR_UNSUPPORTED;
    int st = check_params(L, params);
    if (st) return st;
    for (size_t i = 0; i < L.names.size(); ++i)
        if (!grads[i]) return SRF_ERR_NULL;
    if (m < 0 || dir_div < 1) return SRF_ERR_SHAPE;
    cudaStream_t s = as_stream(stream);
    if (!accumulate) {
        for (size_t i = 0; i < L.names.size(); ++i) {
            auto sh = L.shapes[i];
            size_t n = size_t(sh.first) * (sh.second ? sh.second : 1);
            cudaError_t e = cudaMemsetAsync(grads[i], 0, n * sizeof(float), s);
            if (e != cudaSuccess) {
                set_cuda_error(e);
                return SRF_ERR_CUDA;
            }
        }
    }
    if (m == 0) return SRF_OK;
    if (!workspace) return SRF_ERR_WORKSPACE;
    if (precision == SRF_PRECISION_BF16 || precision == SRF_PRECISION_FP16)
        return mlp_tc_backward(L, params, dsigma, drgb, m, dir_div, grads, workspace, workspace_bytes,
                               precision == SRF_PRECISION_FP16 ? 1 : 0, scaler, s);
    if (precision != SRF_PRECISION_FP32) return SRF_ERR_UNSUPPORTED;
    return mlp_f32_backward(L, params, dsigma, drgb, m, dir_div, grads, workspace, workspace_bytes, s);
}

// ------------------------------------------------------------ generic layer -

extern "C" int srf_linear_forward(float* y, int ldy, const float* x, int ldx, const float* weight, const float* bias,
                                  int64_t max_rows, const int32_t* rows_dev, int n, int k, int act, void* stream) {
    if (!y || !x || !weight) return SRF_ERR_NULL;
    if (max_rows < 0 || n < 1 || k < 1 || ldy < n || ldx < k || act < 0 || act > 2) return SRF_ERR_SHAPE;
    if (max_rows == 0) return SRF_OK;
    return sgemm<true, true>(as_stream(stream), max_rows, n, k, 1, rows_dev, 0, seg1(x, ldx, k), WeightT{weight, k, 0},
                             EpiStore{y, ldy, bias, act});
}

extern "C" int srf_linear_backward(float* dx, int lddx, float* dw, float* db, const float* dy, int lddy,
                                   const float* y, int ldy, const float* x, int ldx, const float* weight,
                                   float* dz_scratch, int64_t max_rows, const int32_t* rows_dev, int n, int k, int act,
                                   int accumulate, void* stream) {
    if (!dy || !dz_scratch || !weight || (act != SRF_ACT_NONE && !y)) return SRF_ERR_NULL;
    if ((dw && !x)) return SRF_ERR_NULL;
    if (max_rows < 0 || n < 1 || k < 1) return SRF_ERR_SHAPE;
    cudaStream_t s = as_stream(stream);
    if (!accumulate) {
        if (dw && cudaMemsetAsync(dw, 0, size_t(n) * k * sizeof(float), s) != cudaSuccess) return SRF_ERR_CUDA;
        if (db && cudaMemsetAsync(db, 0, size_t(n) * sizeof(float), s) != cudaSuccess) return SRF_ERR_CUDA;
    }
    if (max_rows == 0) return SRF_OK;
    int st = SRF_OK;
    // without an activation dz = dy: no pass when the scratch already is dy
    if (!(act == SRF_ACT_NONE && dz_scratch == dy && lddy == n)) {
        act_grad_kernel<<<grid_1d(max_rows * n, 256), 256, 0, s>>>(dz_scratch, n, dy, lddy, y, ldy, max_rows,
                                                                   rows_dev, n, act);
        st = launch_status();
        if (st) return st;
    }
    if (dw) {
        SegRows a = seg1(x, ldx, k);
        a.ones_col = db != nullptr;
        st = sgemm<false, false>(s, n, k + (db ? 1 : 0), max_rows, dw_splits(n, k + 1, max_rows), rows_dev, 1,
                                 ColMajor{dz_scratch, n, 0}, a, EpiAtomicW{dw, k, db, k});
        if (st) return st;
    } else if (db) {
        SegRows a{};
        a.nseg = 0;
        a.ones_col = 1;
        float dummy_unused = 0;
        (void)dummy_unused;
        st = sgemm<false, false>(s, n, 1, max_rows, dw_splits(n, 1, max_rows), rows_dev, 1, ColMajor{dz_scratch, n, 0},
                                 a, EpiAtomicW{nullptr, 0, db, 0});
        if (st) return st;
    }
    if (dx) {
        st = sgemm<true, false>(s, max_rows, k, n, 1, rows_dev, 0, RowMajor{dz_scratch, n, 0}, RowMajor{weight, k, 0},
                                EpiMasked{dx, lddx, nullptr, 0, 0});
        if (st) return st;
    }
    return SRF_OK;
}

extern "C" int srf_positional_encoding_backward(float* dx, const float* x, const float* dout, int ld_dout, int64_t m,
                                                const int32_t* rows_dev, int dims, int degree, void* stream) {
    if (!dx || !x || !dout) return SRF_ERR_NULL;
    if (m < 0 || dims < 1 || degree < 0 || degree > 24 || ld_dout < dims * (2 * degree + 1)) return SRF_ERR_SHAPE;
    if (m == 0) return SRF_OK;
    pe_bwd_kernel<<<grid_1d(m * dims, 256), 256, 0, as_stream(stream)>>>(dx, x, dout, ld_dout, m, rows_dev, dims,
                                                                          degree);
    return launch_status();
}

// PE on rows with a device-side row count (TensoRF renderer input).
int srf_pe_rows(float* out, int64_t ld, const float* x, int64_t m, const int32_t* rows_dev, int dims, int degree,
                cudaStream_t s) {
    pe_rows_kernel<<<grid_1d(m * dims, 256), 256, 0, s>>>(out, ld, x, m, dims, degree, rows_dev);
    return launch_status();
}
