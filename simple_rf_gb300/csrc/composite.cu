// Alpha compositing, forward and adjoint.  One warp per ray; samples are
// processed in rounds of 32 (lane j <-> sample base+j, coalesced), the
// transmittance is a multiplicative warp scan with a carry between rounds, and
// the backward transmittance adjoint is a reverse affine scan.
//
// Formulas follow SimpleNeRF17.py:486-558 (NeRF) and SimpleTensoRF09.py:767-819
// (TensoRF: the extra distance_scale factor).
#include "srf_common.cuh"
#include "tc_primitives.cuh"

namespace srf {
namespace {

constexpr float kEps = 1e-6f;

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct RayCtx {
    const float* sigma;
    const float* z;
    int s;
    float dnorm;
    float ds;
    float inf_depth;
    bool ndc;
    float oz, dz;   // world origin/direction z (NDC depth conversion)
};

// SimpleNeRF17.py:541-558 convert_depth_from_ndc (near = 1).  Every product
// and sum is rounded on its own, as the reference's separate torch ops round
// them (no fused multiply-adds): near z_ndc = 1 the factor 1 / (1 - z_ndc)
// multiplies any rounding difference of the preceding terms.
__device__ __forceinline__ float depth_from_ndc(float zn, float oz, float dz) {
    float tn = -(1.f + oz) / dz;
    float c = zn == 1.f ? 1e-3f : 0.f;
    float a = __fadd_rn(oz, __fmul_rn(tn, dz)) / dz;
    float b = __fsub_rn(1.f / __fadd_rn(__fsub_rn(1.f, zn), c), 1.f);
    return __fadd_rn(__fmul_rn(a, b), tn);
}

// Per-sample quantities of sample i.
__device__ __forceinline__ void sample_terms(const RayCtx& c, int i, float& delta, float& ex, float& alpha,
                                             float& p) {
    float zi = c.z[i];
    float zn = i + 1 < c.s ? c.z[i + 1] : c.inf_depth;
    delta = (zn - zi) * c.dnorm;
    float x = -c.sigma[i] * delta;
    x = x * c.ds;
    ex = expf(x);
    alpha = 1.f - ex;
    p = 1.f - alpha + 1e-10f;
}

// y = sigma delta ds of sample i (the exponent of its 1 - alpha).
__device__ __forceinline__ float sigma_y(const RayCtx& c, int i, float delta) {
    return c.sigma[i] * delta * c.ds;
}

// Pass over the ray storing T (exclusive cumprod of p) and alpha in shared memory.
__device__ void forward_scan(const RayCtx& c, float* sT, float* sA) {
    int lane = threadIdx.x & 31;
    float carry = 1.f;
    for (int base = 0; base < c.s; base += 32) {
        int i = base + lane;
        float delta, ex, alpha, p;
        if (i < c.s) {
            sample_terms(c, i, delta, ex, alpha, p);
        } else {
            alpha = 0.f;
            p = 1.f;
        }
        float inc = p;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            float t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc *= t;
        }
        float exc = __shfl_up_sync(0xffffffffu, inc, 1);
        if (lane == 0) exc = 1.f;
        float T = carry * exc;
        if (i < c.s) {
            sT[i] = T;
            sA[i] = alpha;
        }
        carry = carry * __shfl_sync(0xffffffffu, inc, 31);
    }
    __syncwarp();
}

__device__ __forceinline__ RayCtx make_ctx(const srf_composite_args& a, int r) {
    RayCtx c;
    c.s = a.n_samples;
    c.sigma = a.sigma + int64_t(r) * c.s;
    c.z = a.z + int64_t(r) * c.s;
    c.ndc = (a.flags & SRF_COMPOSITE_NDC) != 0;
    const float* dv = c.ndc ? a.rays_d_ndc + 3 * r : a.rays_d + 3 * r;
    c.dnorm = sqrtf(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
    c.ds = a.distance_scale;
    c.inf_depth = c.ndc ? 1.f : 1e10f;
    c.oz = c.ndc ? a.rays_o[3 * r + 2] : 0.f;
    c.dz = c.ndc ? a.rays_d[3 * r + 2] : 0.f;
    return c;
}

__device__ __forceinline__ bool white_for(const srf_composite_args& a, int r) {
    return (a.flags & SRF_COMPOSITE_WHITE_BKGD) || (a.white_per_ray && a.white_per_ray[r]);
}

// A training loss folded into compositing (srf_composite_loss): the rgb term
// rgb_scale sum_c (rgb_c - t_c)^2 (MSE14.compute_mse with rgb_scale = 1 / (3 N)),
// the depth term depth_scale |depth - t| or depth_scale (depth - t)^2 on masked
// rays, and MassConcentrationLoss06's mc_scale sum_b -x_b ln x_b with x_b the
// bin sums of the weights + 1e-3.
struct LossArgs {
    const float* target_rgb;
    float rgb_scale;
    const float* target_depth;
    const uint8_t* depth_mask;
    float depth_scale;
    int depth_squared;
    BinLayout bins;   // bins.nb == 0: no entropy term
    const uint8_t* mc_mask;
    float mc_scale;
    float* loss;
};

__device__ __forceinline__ bool depth_term(const LossArgs& L, int r) {
    return L.target_depth && (!L.depth_mask || L.depth_mask[r]);
}

__device__ __forceinline__ bool mc_term(const LossArgs& L, int r) {
    return L.bins.nb > 0 && (!L.mc_mask || L.mc_mask[r]);
}

// Sum over the ray's samples of bin b of v (lane j holds samples j + 32 k).
template <int R>
__device__ __forceinline__ float bin_sum(const float (&v)[R], const BinLayout& bl, int b, int lane) {
    float part = 0.f;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int i = 32 * k + lane;
        if (i >= bl.start[b] && i < bl.start[b + 1]) part += v[k];
    }
    return warp_sum(part);
}


__global__ void composite_fwd_kernel(srf_composite_args a) {
    extern __shared__ float smem[];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int r = blockIdx.x * (blockDim.x >> 5) + warp;
    if (r >= a.n_rays) return;
    float* sT = smem + size_t(warp) * 2 * a.n_samples;
    float* sA = sT + a.n_samples;
    RayCtx c = make_ctx(a, r);
    forward_scan(c, sT, sA);
    const float* rgb = a.rgb ? a.rgb + int64_t(r) * c.s * 3 : nullptr;   // NULL: zero colours
    float cr = 0.f, cg = 0.f, cb = 0.f, acc = 0.f, wz = 0.f, wzn = 0.f;
    for (int i = lane; i < c.s; i += 32) {
        float w = sA[i] * sT[i];
        if (rgb) {
            cr += w * rgb[3 * i];
            cg += w * rgb[3 * i + 1];
            cb += w * rgb[3 * i + 2];
        }
        acc += w;
        float zi = c.z[i];
        if (c.ndc) {
            wzn += w * zi;
            wz += w * depth_from_ndc(zi, c.oz, c.dz);
        } else {
            wz += w * zi;
        }
    }
    cr = warp_sum(cr); cg = warp_sum(cg); cb = warp_sum(cb);
    acc = warp_sum(acc); wz = warp_sum(wz); wzn = warp_sum(wzn);
    float depth = wz / (acc + kEps);
    float depth_ndc = wzn / (acc + kEps);
    float var = 0.f, var_ndc = 0.f;
    int64_t ro = int64_t(r) * c.s;
    for (int i = lane; i < c.s; i += 32) {
        float w = sA[i] * sT[i];
        float zi = c.z[i];
        float zm = c.ndc ? depth_from_ndc(zi, c.oz, c.dz) : zi;
        float d = zm - depth;
        var += w * (d * d);
        if (c.ndc) {
            float dn = zi - depth_ndc;
            var_ndc += w * (dn * dn);
        }
        if (a.alpha) a.alpha[ro + i] = sA[i];
        if (a.visibility) a.visibility[ro + i] = sT[i];
        if (a.weights) a.weights[ro + i] = w;
    }
    var = warp_sum(var);
    var_ndc = warp_sum(var_ndc);
    if (lane == 0) {
        if (white_for(a, r)) {
            cr = cr + (1.f - acc);
            cg = cg + (1.f - acc);
            cb = cb + (1.f - acc);
        }
        if (a.rgb_map) {
            a.rgb_map[3 * r] = cr;
            a.rgb_map[3 * r + 1] = cg;
            a.rgb_map[3 * r + 2] = cb;
        }
        if (a.acc) a.acc[r] = acc;
        if (a.depth) a.depth[r] = depth;
        if (a.depth_var) a.depth_var[r] = var;
        if (c.ndc) {
            if (a.depth_ndc) a.depth_ndc[r] = depth_ndc;
            if (a.depth_var_ndc) a.depth_var_ndc[r] = var_ndc;
        }
    }
}

__global__ void composite_bwd_kernel(srf_composite_args a) {
    extern __shared__ float smem[];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int r = blockIdx.x * (blockDim.x >> 5) + warp;
    if (r >= a.n_rays) return;
    float* sT = smem + size_t(warp) * 2 * a.n_samples;
    float* sA = sT + a.n_samples;
    RayCtx c = make_ctx(a, r);
    forward_scan(c, sT, sA);
    const float* rgb = a.rgb ? a.rgb + int64_t(r) * c.s * 3 : nullptr;
    // forward sums: acc, depth (and NDC depth)
    float acc = 0.f, wz = 0.f, wzn = 0.f;
    for (int i = lane; i < c.s; i += 32) {
        float w = sA[i] * sT[i];
        acc += w;
        float zi = c.z[i];
        if (c.ndc) {
            wzn += w * zi;
            wz += w * depth_from_ndc(zi, c.oz, c.dz);
        } else {
            wz += w * zi;
        }
    }
    acc = warp_sum(acc); wz = warp_sum(wz); wzn = warp_sum(wzn);
    float inv = 1.f / (acc + kEps);
    float depth = wz / (acc + kEps), depth_ndc = wzn / (acc + kEps);
    float gd = a.g_depth ? a.g_depth[r] : 0.f;
    float gv = a.g_depth_var ? a.g_depth_var[r] : 0.f;
    float gdn = (c.ndc && a.g_depth_ndc) ? a.g_depth_ndc[r] : 0.f;
    float gvn = (c.ndc && a.g_depth_var_ndc) ? a.g_depth_var_ndc[r] : 0.f;
    // B = sum w (z - depth): the depth_var gradient's coupling term
    float bsum = 0.f, bsum_n = 0.f;
    if (gv != 0.f || gvn != 0.f) {
        for (int i = lane; i < c.s; i += 32) {
            float w = sA[i] * sT[i];
            float zi = c.z[i];
            float zm = c.ndc ? depth_from_ndc(zi, c.oz, c.dz) : zi;
            bsum += w * (zm - depth);
            if (c.ndc) bsum_n += w * (zi - depth_ndc);
        }
        bsum = warp_sum(bsum);
        bsum_n = warp_sum(bsum_n);
    }
    float g0 = 0.f, g1 = 0.f, g2 = 0.f;
    if (a.g_rgb) {
        g0 = a.g_rgb[3 * r];
        g1 = a.g_rgb[3 * r + 1];
        g2 = a.g_rgb[3 * r + 2];
    }
    float gacc = a.g_acc ? a.g_acc[r] : 0.f;
    if (white_for(a, r)) gacc -= g0 + g1 + g2;
    int64_t ro = int64_t(r) * c.s;
    // dL/dw_i
    auto G_of = [&](int i) -> float {
        float zi = c.z[i];
        float zm = c.ndc ? depth_from_ndc(zi, c.oz, c.dz) : zi;
        float g = (rgb ? rgb[3 * i] * g0 + rgb[3 * i + 1] * g1 + rgb[3 * i + 2] * g2 : 0.f) + gacc;
        if (a.g_weights) g += a.g_weights[ro + i];
        float d = zm - depth;
        g += gd * d * inv + gv * (d * d - 2.f * bsum * d * inv);
        if (c.ndc) {
            float dn = zi - depth_ndc;
            g += gdn * dn * inv + gvn * (dn * dn - 2.f * bsum_n * dn * inv);
        }
        return g;
    };
    // reverse affine scan: R_i = G_{i+1} a_{i+1} + p_{i+1} R_{i+1}, R_{S-1} = 0
    float carry = 0.f;                  // R at the first sample of the round to the right
    float next_ga = 0.f, next_p = 0.f;  // G*alpha and p of that first sample
    int last_base = ((c.s - 1) / 32) * 32;
    for (int base = last_base; base >= 0; base -= 32) {
        int i = base + lane;
        bool in = i < c.s;
        float Gi = 0.f, alpha = 0.f, T = 0.f, p = 1.f, ga = 0.f;
        if (in) {
            Gi = G_of(i);
            alpha = sA[i];
            T = sT[i];
            p = 1.f - alpha + 1e-10f;
            ga = Gi * alpha;
        }
        // coefficients of sample i: a_i = G_{i+1} alpha_{i+1}, b_i = p_{i+1}
        float ga_next = __shfl_down_sync(0xffffffffu, ga, 1);
        float p_next = __shfl_down_sync(0xffffffffu, p, 1);
        if (lane == 31) {
            ga_next = next_ga;
            p_next = next_p;
        }
        float A = in && i + 1 < c.s ? ga_next : 0.f;
        float B = in && i + 1 < c.s ? p_next : 0.f;
        // inclusive suffix composition of the affine maps lane..31
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            float A2 = __shfl_down_sync(0xffffffffu, A, o);
            float B2 = __shfl_down_sync(0xffffffffu, B, o);
            if (lane + o < 32) {
                A = A + B * A2;
                B = B * B2;
            }
        }
        float R = A + B * carry;
        if (in) {
            float dalpha = T * (Gi - R);
            float delta, ex, al, pp;
            sample_terms(c, i, delta, ex, al, pp);
            float dx = -dalpha * ex;
            dx = dx * c.ds;
            a.d_sigma[ro + i] = -dx * delta;
            if (a.d_rgb) {
                float w = alpha * T;
                float* dr = a.d_rgb + (ro + i) * 3;
                dr[0] = w * g0;
                dr[1] = w * g1;
                dr[2] = w * g2;
            }
        }
        carry = __shfl_sync(0xffffffffu, R, 0);
        next_ga = __shfl_sync(0xffffffffu, ga, 0);
        next_p = __shfl_sync(0xffffffffu, p, 0);
    }
}

// ---------------------------------------------------------------------------
// Register-resident variants for rays of at most 32 * R samples (R <= 8: every
// NeRF configuration, 64 / 128 / 192 / 256 samples).  Lane j holds samples
// j, j + 32, ..., j + 32 (R - 1) in registers: every global load of the ray is
// issued before the first scan step (the per-round loads of the shared-memory
// kernels wait for the previous round's scan), and the R rounds' scans only
// chain through one carry.  Arithmetic, and the order of every product and sum,
// are those of the shared-memory kernels, so the outputs are identical.
// ---------------------------------------------------------------------------

template <int R>
__device__ __forceinline__ void scan_rounds(float (&T)[R], int lane) {
    float carry = 1.f;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        float inc = T[k];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            float t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc *= t;
        }
        float exc = __shfl_up_sync(0xffffffffu, inc, 1);
        if (lane == 0) exc = 1.f;
        T[k] = carry * exc;
        carry = carry * __shfl_sync(0xffffffffu, inc, 31);
    }
}

// Exp-of-prefix-sum transmittance: on entry Y[k] holds y = sigma delta ds of
// each sample; on exit it holds T = exp(-(sum of y over the earlier samples)).
template <int R>
__device__ __forceinline__ void exp_scan_rounds(float (&Y)[R], int lane) {
    float carry = 0.f;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        float inc = Y[k];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            float t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        float exc = __shfl_up_sync(0xffffffffu, inc, 1);
        if (lane == 0) exc = 0.f;
        Y[k] = expf(-(carry + exc));
        carry = carry + __shfl_sync(0xffffffffu, inc, 31);
    }
}

// One ray of the forward (lane j holds samples j, j + 32, ...): c's sigma / z and
// rgb may point at global memory or at a shared-memory copy of the ray.
template <int R, bool LOSS>
__device__ __forceinline__ void fwd_ray(const srf_composite_args& a, const LossArgs& L, int r, RayCtx c,
                                        const float* rgb) {
    const int lane = threadIdx.x & 31;
    const bool exp_prefix = (a.flags & SRF_COMPOSITE_EXP_PREFIX) != 0;
    float al[R], T[R], zz[R], c0[R], c1[R], c2[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int i = 32 * k + lane;
        al[k] = 0.f;
        T[k] = 1.f;
        zz[k] = 0.f;
        c0[k] = c1[k] = c2[k] = 0.f;
        if (i < c.s) {
            float delta, ex, alpha, p;
            sample_terms(c, i, delta, ex, alpha, p);
            al[k] = alpha;
            T[k] = exp_prefix ? sigma_y(c, i, delta) : p;
            zz[k] = c.z[i];
            if (rgb) {
                c0[k] = rgb[3 * i];
                c1[k] = rgb[3 * i + 1];
                c2[k] = rgb[3 * i + 2];
            }
        } else if (exp_prefix) {
            T[k] = 0.f;
        }
    }
    if (exp_prefix)
        exp_scan_rounds<R>(T, lane);
    else
        scan_rounds<R>(T, lane);
    float cr = 0.f, cg = 0.f, cb = 0.f, acc = 0.f, wz = 0.f, wzn = 0.f;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (32 * k + lane < c.s) {
            float w = al[k] * T[k];
            if (rgb) {
                cr += w * c0[k];
                cg += w * c1[k];
                cb += w * c2[k];
            }
            acc += w;
            if (c.ndc) {
                wzn += w * zz[k];
                wz += w * depth_from_ndc(zz[k], c.oz, c.dz);
            } else {
                wz += w * zz[k];
            }
        }
    }
    cr = warp_sum(cr); cg = warp_sum(cg); cb = warp_sum(cb);
    acc = warp_sum(acc); wz = warp_sum(wz); wzn = warp_sum(wzn);
    float depth = wz / (acc + kEps);
    float depth_ndc = wzn / (acc + kEps);
    float var = 0.f, var_ndc = 0.f;
    int64_t ro = int64_t(r) * c.s;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int i = 32 * k + lane;
        if (i < c.s) {
            float w = al[k] * T[k];
            float zm = c.ndc ? depth_from_ndc(zz[k], c.oz, c.dz) : zz[k];
            float d = zm - depth;
            var += w * (d * d);
            if (c.ndc) {
                float dn = zz[k] - depth_ndc;
                var_ndc += w * (dn * dn);
            }
            if (a.alpha) a.alpha[ro + i] = al[k];
            if (a.visibility) a.visibility[ro + i] = T[k];
            if (a.weights) a.weights[ro + i] = w;
        }
    }
    var = warp_sum(var);
    var_ndc = warp_sum(var_ndc);
    float lray = 0.f;
    if (LOSS && mc_term(L, r)) {
        float w[R];
#pragma unroll
        for (int k = 0; k < R; ++k) w[k] = 32 * k + lane < c.s ? al[k] * T[k] : 0.f;
        for (int b = 0; b < L.bins.nb; ++b) {
            const float x = bin_sum<R>(w, L.bins, b, lane) + 1e-3f;
            lray -= x * logf(x);
        }
        lray *= L.mc_scale;
    }
    if (lane == 0) {
        if (white_for(a, r)) {
            cr = cr + (1.f - acc);
            cg = cg + (1.f - acc);
            cb = cb + (1.f - acc);
        }
        if (LOSS) {
            if (L.target_rgb) {
                const float e0 = cr - L.target_rgb[3 * r], e1 = cg - L.target_rgb[3 * r + 1],
                            e2 = cb - L.target_rgb[3 * r + 2];
                lray += L.rgb_scale * (e0 * e0 + e1 * e1 + e2 * e2);
            }
            if (depth_term(L, r)) {
                const float e = depth - L.target_depth[r];
                lray += L.depth_scale * (L.depth_squared ? e * e : fabsf(e));
            }
            atomicAdd(L.loss, lray);
        }
        if (a.rgb_map) {
            a.rgb_map[3 * r] = cr;
            a.rgb_map[3 * r + 1] = cg;
            a.rgb_map[3 * r + 2] = cb;
        }
        if (a.acc) a.acc[r] = acc;
        if (a.depth) a.depth[r] = depth;
        if (a.depth_var) a.depth_var[r] = var;
        if (c.ndc) {
            if (a.depth_ndc) a.depth_ndc[r] = depth_ndc;
            if (a.depth_var_ndc) a.depth_var_ndc[r] = var_ndc;
        }
    }
}

template <int R, bool LOSS>
__global__ void __launch_bounds__(256) composite_fwd_reg_kernel(srf_composite_args a, LossArgs L) {
    int warp = threadIdx.x >> 5;
    int r = blockIdx.x * (blockDim.x >> 5) + warp;
    if (r >= a.n_rays) return;
    RayCtx c = make_ctx(a, r);
    fwd_ray<R, LOSS>(a, L, r, c, a.rgb ? a.rgb + int64_t(r) * c.s * 3 : nullptr);   // NULL: zero colours
}

// One ray of the adjoint; sigma / z / rgb as in fwd_ray.
template <int R, bool LOSS>
__device__ __forceinline__ void bwd_ray(const srf_composite_args& a, const LossArgs& L, int r, RayCtx c,
                                        const float* rgb) {
    const int lane = threadIdx.x & 31;
    const bool exp_prefix = (a.flags & SRF_COMPOSITE_EXP_PREFIX) != 0;
    const int64_t ro = int64_t(r) * c.s;
    // G holds dL/dw_i once formed; until then the colour dot product's partial terms
    float al[R], T[R], ex_[R], dl[R], zz[R], G[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int i = 32 * k + lane;
        al[k] = 0.f;
        T[k] = 1.f;
        ex_[k] = dl[k] = zz[k] = G[k] = 0.f;
        if (i < c.s) {
            float delta, ex, alpha, p;
            sample_terms(c, i, delta, ex, alpha, p);
            al[k] = alpha;
            T[k] = exp_prefix ? sigma_y(c, i, delta) : p;
            ex_[k] = ex;
            dl[k] = delta;
            zz[k] = c.z[i];
            if (a.g_weights) G[k] = a.g_weights[ro + i];
        }
    }
    float g0 = 0.f, g1 = 0.f, g2 = 0.f;
    if (a.g_rgb) {
        g0 = a.g_rgb[3 * r];
        g1 = a.g_rgb[3 * r + 1];
        g2 = a.g_rgb[3 * r + 2];
    }
    float gacc = a.g_acc ? a.g_acc[r] : 0.f;
    // colour terms of G (the loads stay off the scan's dependency chain); with a
    // loss the colours stay in registers until the loss gradient of rgb is known
    float cdot[R], c0[LOSS ? R : 1], c1[LOSS ? R : 1], c2[LOSS ? R : 1];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int i = 32 * k + lane;
        if (LOSS) {
            const bool in = rgb && i < c.s;
            c0[k] = in ? rgb[3 * i] : 0.f;
            c1[k] = in ? rgb[3 * i + 1] : 0.f;
            c2[k] = in ? rgb[3 * i + 2] : 0.f;
        } else {
            cdot[k] = (rgb && i < c.s) ? rgb[3 * i] * g0 + rgb[3 * i + 1] * g1 + rgb[3 * i + 2] * g2 : 0.f;
        }
        if (exp_prefix && i >= c.s) T[k] = 0.f;
    }
    if (exp_prefix)
        exp_scan_rounds<R>(T, lane);
    else
        scan_rounds<R>(T, lane);
    float acc = 0.f, wz = 0.f, wzn = 0.f;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (32 * k + lane < c.s) {
            float w = al[k] * T[k];
            acc += w;
            if (c.ndc) {
                wzn += w * zz[k];
                wz += w * depth_from_ndc(zz[k], c.oz, c.dz);
            } else {
                wz += w * zz[k];
            }
        }
    }
    acc = warp_sum(acc); wz = warp_sum(wz); wzn = warp_sum(wzn);
    float inv = 1.f / (acc + kEps);
    float depth = wz / (acc + kEps), depth_ndc = wzn / (acc + kEps);
    float gd = a.g_depth ? a.g_depth[r] : 0.f;
    if (LOSS) {
        // the loss gradient of this ray's outputs, from the recomputed forward
        if (L.target_rgb) {
            float cr = 0.f, cg = 0.f, cb = 0.f;
#pragma unroll
            for (int k = 0; k < R; ++k) {
                if (32 * k + lane < c.s) {
                    const float w = al[k] * T[k];
                    cr += w * c0[k];
                    cg += w * c1[k];
                    cb += w * c2[k];
                }
            }
            cr = warp_sum(cr); cg = warp_sum(cg); cb = warp_sum(cb);
            if (white_for(a, r)) {
                cr = cr + (1.f - acc);
                cg = cg + (1.f - acc);
                cb = cb + (1.f - acc);
            }
            const float s2 = 2.f * L.rgb_scale;
            g0 += s2 * (cr - L.target_rgb[3 * r]);
            g1 += s2 * (cg - L.target_rgb[3 * r + 1]);
            g2 += s2 * (cb - L.target_rgb[3 * r + 2]);
        }
        if (depth_term(L, r)) {
            const float e = depth - L.target_depth[r];
            gd += L.depth_squared ? 2.f * L.depth_scale * e
                                  : L.depth_scale * (e > 0.f ? 1.f : (e < 0.f ? -1.f : 0.f));
        }
        if (mc_term(L, r)) {
            float w[R];
#pragma unroll
            for (int k = 0; k < R; ++k) w[k] = 32 * k + lane < c.s ? al[k] * T[k] : 0.f;
            for (int b = 0; b < L.bins.nb; ++b) {
                const float x = bin_sum<R>(w, L.bins, b, lane) + 1e-3f;
                const float gb = -(logf(x) + 1.f) * L.mc_scale;
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    const int i = 32 * k + lane;
                    if (i >= L.bins.start[b] && i < L.bins.start[b + 1]) G[k] += gb;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < R; ++k) cdot[k] = c0[k] * g0 + c1[k] * g1 + c2[k] * g2;
    }
    if (white_for(a, r)) gacc -= g0 + g1 + g2;
    float gv = a.g_depth_var ? a.g_depth_var[r] : 0.f;
    float gdn = (c.ndc && a.g_depth_ndc) ? a.g_depth_ndc[r] : 0.f;
    float gvn = (c.ndc && a.g_depth_var_ndc) ? a.g_depth_var_ndc[r] : 0.f;
    float bsum = 0.f, bsum_n = 0.f;
    if (gv != 0.f || gvn != 0.f) {
#pragma unroll
        for (int k = 0; k < R; ++k) {
            if (32 * k + lane < c.s) {
                float w = al[k] * T[k];
                float zm = c.ndc ? depth_from_ndc(zz[k], c.oz, c.dz) : zz[k];
                bsum += w * (zm - depth);
                if (c.ndc) bsum_n += w * (zz[k] - depth_ndc);
            }
        }
        bsum = warp_sum(bsum);
        bsum_n = warp_sum(bsum_n);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        float zm = c.ndc ? depth_from_ndc(zz[k], c.oz, c.dz) : zz[k];
        float g = cdot[k] + gacc;
        if (a.g_weights || (LOSS && mc_term(L, r))) g += G[k];
        float d = zm - depth;
        g += gd * d * inv + gv * (d * d - 2.f * bsum * d * inv);
        if (c.ndc) {
            float dn = zz[k] - depth_ndc;
            g += gdn * dn * inv + gvn * (dn * dn - 2.f * bsum_n * dn * inv);
        }
        G[k] = g;
    }
    if (exp_prefix) {
        // w_i = (1 - e^{-y_i}) T_i with T_i = exp(-sum_{j<i} y_j):
        // dL/dy_k = G_k e^{-y_k} T_k - sum_{i>k} G_i w_i (a reverse exclusive sum scan)
        float carry = 0.f;
#pragma unroll
        for (int k = R - 1; k >= 0; --k) {
            const int i = 32 * k + lane;
            if (32 * k >= c.s) continue;   // warp-uniform
            const bool in = i < c.s;
            const float w = in ? al[k] * T[k] : 0.f;
            const float gw = in ? G[k] * w : 0.f;
            float inc = gw;   // inclusive suffix sum over lanes lane..31 of this round
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                float t = __shfl_down_sync(0xffffffffu, inc, o);
                if (lane + o < 32) inc += t;
            }
            const float after = carry + (inc - gw);   // sum over the samples after i
            if (in) {
                const float dy = G[k] * ex_[k] * T[k] - after;
                a.d_sigma[ro + i] = dy * c.ds * dl[k];
                if (a.d_rgb) {
                    float* dr = a.d_rgb + (ro + i) * 3;
                    dr[0] = w * g0;
                    dr[1] = w * g1;
                    dr[2] = w * g2;
                }
            }
            carry = carry + __shfl_sync(0xffffffffu, inc, 0);
        }
        return;
    }
    // reverse affine scan: R_i = G_{i+1} a_{i+1} + p_{i+1} R_{i+1}, R_{S-1} = 0
    float carry = 0.f, next_ga = 0.f, next_p = 0.f;
#pragma unroll
    for (int k = R - 1; k >= 0; --k) {
        const int i = 32 * k + lane;
        if (32 * k >= c.s) continue;   // warp-uniform: rounds past the ray's end
        bool in = i < c.s;
        float Gi = in ? G[k] : 0.f, alpha = in ? al[k] : 0.f, Tk = in ? T[k] : 0.f;
        float p = in ? 1.f - alpha + 1e-10f : 1.f;
        float ga = Gi * alpha;
        float ga_next = __shfl_down_sync(0xffffffffu, ga, 1);
        float p_next = __shfl_down_sync(0xffffffffu, p, 1);
        if (lane == 31) {
            ga_next = next_ga;
            p_next = next_p;
        }
        float A = in && i + 1 < c.s ? ga_next : 0.f;
        float B = in && i + 1 < c.s ? p_next : 0.f;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            float A2 = __shfl_down_sync(0xffffffffu, A, o);
            float B2 = __shfl_down_sync(0xffffffffu, B, o);
            if (lane + o < 32) {
                A = A + B * A2;
                B = B * B2;
            }
        }
        float Rr = A + B * carry;
        if (in) {
            float dalpha = Tk * (Gi - Rr);
            float dx = -dalpha * ex_[k];
            dx = dx * c.ds;
            a.d_sigma[ro + i] = -dx * dl[k];
            if (a.d_rgb) {
                float w = alpha * Tk;
                float* dr = a.d_rgb + (ro + i) * 3;
                dr[0] = w * g0;
                dr[1] = w * g1;
                dr[2] = w * g2;
            }
        }
        carry = __shfl_sync(0xffffffffu, Rr, 0);
        next_ga = __shfl_sync(0xffffffffu, ga, 0);
        next_p = __shfl_sync(0xffffffffu, p, 0);
    }
}

template <int R, bool LOSS>
__global__ void __launch_bounds__(256) composite_bwd_reg_kernel(srf_composite_args a, LossArgs L) {
    int warp = threadIdx.x >> 5;
    int r = blockIdx.x * (blockDim.x >> 5) + warp;
    if (r >= a.n_rays) return;
    RayCtx c = make_ctx(a, r);
    bwd_ray<R, LOSS>(a, L, r, c, a.rgb ? a.rgb + int64_t(r) * c.s * 3 : nullptr);
}

// ---------------------------------------------------------------------------
// Blocked per-ray bodies for the staged kernels: lane j owns the R contiguous
// samples R j .. R j + R - 1 of a ray held in shared memory (R even, S % 4 == 0,
// 16-byte aligned rows), so a scan over the ray is R sequential steps in each lane
// plus one warp scan of the lanes' totals (instead of a warp scan per 32-sample
// round), and the loads are 8-byte vectors.  The arithmetic of each sample is that
// of fwd_ray / bwd_ray; the scans and sums group the products and sums
// differently.  The per-sample outputs (weights; d_sigma and d_rgb) go into the
// ray's shared-memory stage, which the caller stores with bulk copies.
// ---------------------------------------------------------------------------

// On entry T[k] = p of sample R lane + k; on exit the product of p over the ray's
// earlier samples.
template <int R>
__device__ __forceinline__ void scan_blk(float (&T)[R], int lane) {
    float run = 1.f, ex[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        ex[k] = run;
        run *= T[k];
    }
    float inc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc *= t;
    }
    float pre = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane == 0) pre = 1.f;
#pragma unroll
    for (int k = 0; k < R; ++k) T[k] = pre * ex[k];
}

// On entry Y[k] = y = sigma delta ds of sample R lane + k; on exit T = exp(-(sum
// of y over the earlier samples)).
template <int R>
__device__ __forceinline__ void exp_scan_blk(float (&Y)[R], int lane) {
    float run = 0.f, ex[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        ex[k] = run;
        run += Y[k];
    }
    float inc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    float pre = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane == 0) pre = 0.f;
#pragma unroll
    for (int k = 0; k < R; ++k) Y[k] = expf(-(pre + ex[k]));
}

template <int R>
__device__ __forceinline__ float bin_sum_blk(const float (&v)[R], const BinLayout& bl, int b, int lane) {
    float part = 0.f;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int i = R * lane + k;
        if (i >= bl.start[b] && i < bl.start[b + 1]) part += v[k];
    }
    return warp_sum(part);
}

// This lane's sigma, z and rgb from the stage, and the z of the sample after its
// block (a pair of samples is wholly inside the ray or wholly past its end).
template <int R>
__device__ __forceinline__ void load_blk(const RayCtx& c, const float* rgb, int i0, float (&sg)[R], float (&zz)[R],
                                         float (&c0)[R], float (&c1)[R], float (&c2)[R], float& zlast) {
#pragma unroll
    for (int k = 0; k < R; k += 2) {
        const int i = i0 + k;
        float2 s2 = make_float2(0.f, 0.f), z2 = s2, r0 = s2, r1 = s2, r2 = s2;
        if (i < c.s) {
            s2 = *reinterpret_cast<const float2*>(c.sigma + i);
            z2 = *reinterpret_cast<const float2*>(c.z + i);
            if (rgb) {
                const float2* pr = reinterpret_cast<const float2*>(rgb + 3 * i);
                r0 = pr[0];
                r1 = pr[1];
                r2 = pr[2];
            }
        }
        sg[k] = s2.x; sg[k + 1] = s2.y;
        zz[k] = z2.x; zz[k + 1] = z2.y;
        c0[k] = r0.x; c1[k] = r0.y; c2[k] = r1.x;
        c0[k + 1] = r1.y; c1[k + 1] = r2.x; c2[k + 1] = r2.y;
    }
    zlast = i0 + R < c.s ? c.z[i0 + R] : c.inf_depth;
}

// delta, e^x, alpha and the scan input of sample k of the block (sample_terms).
template <int R>
__device__ __forceinline__ void terms_blk(const RayCtx& c, bool exp_prefix, int i0, const float (&sg)[R],
                                          const float (&zz)[R], float zlast, float (&al)[R], float (&T)[R],
                                          float (&ex_)[R], float (&dl)[R]) {
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int i = i0 + k;
        al[k] = 0.f;
        T[k] = exp_prefix ? 0.f : 1.f;
        ex_[k] = dl[k] = 0.f;
        if (i < c.s) {
            const float zn = k + 1 < R ? (i + 1 < c.s ? zz[k + 1] : c.inf_depth) : zlast;
            const float delta = (zn - zz[k]) * c.dnorm;
            float x = -sg[k] * delta;
            x = x * c.ds;
            const float ex = expf(x);
            al[k] = 1.f - ex;
            T[k] = exp_prefix ? sg[k] * delta * c.ds : 1.f - al[k] + 1e-10f;
            ex_[k] = ex;
            dl[k] = delta;
        }
    }
}

template <int R, bool LOSS>
__device__ __forceinline__ void fwd_ray_blk(const srf_composite_args& a, const LossArgs& L, int r, RayCtx c,
                                            const float* rgb, float* wout) {
    const int lane = threadIdx.x & 31;
    const int i0 = R * lane;
    const bool exp_prefix = (a.flags & SRF_COMPOSITE_EXP_PREFIX) != 0;
    float sg[R], zz[R], c0[R], c1[R], c2[R], al[R], T[R], ex_[R], dl[R], zlast;
    load_blk<R>(c, rgb, i0, sg, zz, c0, c1, c2, zlast);
    terms_blk<R>(c, exp_prefix, i0, sg, zz, zlast, al, T, ex_, dl);
    if (exp_prefix)
        exp_scan_blk<R>(T, lane);
    else
        scan_blk<R>(T, lane);
    float cr = 0.f, cg = 0.f, cb = 0.f, acc = 0.f, wz = 0.f, wzn = 0.f;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (i0 + k < c.s) {
            const float w = al[k] * T[k];
            if (rgb) {
                cr += w * c0[k];
                cg += w * c1[k];
                cb += w * c2[k];
            }
            acc += w;
            if (c.ndc) {
                wzn += w * zz[k];
                wz += w * depth_from_ndc(zz[k], c.oz, c.dz);
            } else {
                wz += w * zz[k];
            }
        }
    }
    cr = warp_sum(cr); cg = warp_sum(cg); cb = warp_sum(cb);
    acc = warp_sum(acc); wz = warp_sum(wz); wzn = warp_sum(wzn);
    const float depth = wz / (acc + kEps);
    const float depth_ndc = wzn / (acc + kEps);
    float var = 0.f, var_ndc = 0.f;
    const int64_t ro = int64_t(r) * c.s;
    __syncwarp();   // every lane has read its stage rows before the weights overwrite sigma
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int i = i0 + k;
        if (i < c.s) {
            const float w = al[k] * T[k];
            const float zm = c.ndc ? depth_from_ndc(zz[k], c.oz, c.dz) : zz[k];
            const float d = zm - depth;
            var += w * (d * d);
            if (c.ndc) {
                const float dn = zz[k] - depth_ndc;
                var_ndc += w * (dn * dn);
            }
            if (a.alpha) a.alpha[ro + i] = al[k];
            if (a.visibility) a.visibility[ro + i] = T[k];
            if (a.weights) wout[i] = w;
        }
    }
    var = warp_sum(var);
    var_ndc = warp_sum(var_ndc);
    float lray = 0.f;
    if (LOSS && mc_term(L, r)) {
        float w[R];
#pragma unroll
        for (int k = 0; k < R; ++k) w[k] = i0 + k < c.s ? al[k] * T[k] : 0.f;
        for (int b = 0; b < L.bins.nb; ++b) {
            const float x = bin_sum_blk<R>(w, L.bins, b, lane) + 1e-3f;
            lray -= x * logf(x);
        }
        lray *= L.mc_scale;
    }
    if (lane == 0) {
        if (white_for(a, r)) {
            cr = cr + (1.f - acc);
            cg = cg + (1.f - acc);
            cb = cb + (1.f - acc);
        }
        if (LOSS) {
            if (L.target_rgb) {
                const float e0 = cr - L.target_rgb[3 * r], e1 = cg - L.target_rgb[3 * r + 1],
                            e2 = cb - L.target_rgb[3 * r + 2];
                lray += L.rgb_scale * (e0 * e0 + e1 * e1 + e2 * e2);
            }
            if (depth_term(L, r)) {
                const float e = depth - L.target_depth[r];
                lray += L.depth_scale * (L.depth_squared ? e * e : fabsf(e));
            }
            atomicAdd(L.loss, lray);
        }
        if (a.rgb_map) {
            a.rgb_map[3 * r] = cr;
            a.rgb_map[3 * r + 1] = cg;
            a.rgb_map[3 * r + 2] = cb;
        }
        if (a.acc) a.acc[r] = acc;
        if (a.depth) a.depth[r] = depth;
        if (a.depth_var) a.depth_var[r] = var;
        if (c.ndc) {
            if (a.depth_ndc) a.depth_ndc[r] = depth_ndc;
            if (a.depth_var_ndc) a.depth_var_ndc[r] = var_ndc;
        }
    }
}

template <int R, bool LOSS>
__device__ __forceinline__ void bwd_ray_blk(const srf_composite_args& a, const LossArgs& L, int r, RayCtx c,
                                            const float* rgb, float* dsig_out, float* drgb_out) {
    const int lane = threadIdx.x & 31;
    const int i0 = R * lane;
    const bool exp_prefix = (a.flags & SRF_COMPOSITE_EXP_PREFIX) != 0;
    const int64_t ro = int64_t(r) * c.s;
    float sg[R], zz[R], c0[R], c1[R], c2[R], al[R], T[R], ex_[R], dl[R], G[R], zlast;
    load_blk<R>(c, rgb, i0, sg, zz, c0, c1, c2, zlast);
    terms_blk<R>(c, exp_prefix, i0, sg, zz, zlast, al, T, ex_, dl);
#pragma unroll
    for (int k = 0; k < R; ++k) G[k] = (a.g_weights && i0 + k < c.s) ? a.g_weights[ro + i0 + k] : 0.f;
    float g0 = 0.f, g1 = 0.f, g2 = 0.f;
    if (a.g_rgb) {
        g0 = a.g_rgb[3 * r];
        g1 = a.g_rgb[3 * r + 1];
        g2 = a.g_rgb[3 * r + 2];
    }
    float gacc = a.g_acc ? a.g_acc[r] : 0.f;
    if (exp_prefix)
        exp_scan_blk<R>(T, lane);
    else
        scan_blk<R>(T, lane);
    float acc = 0.f, wz = 0.f, wzn = 0.f;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (i0 + k < c.s) {
            const float w = al[k] * T[k];
            acc += w;
            if (c.ndc) {
                wzn += w * zz[k];
                wz += w * depth_from_ndc(zz[k], c.oz, c.dz);
            } else {
                wz += w * zz[k];
            }
        }
    }
    acc = warp_sum(acc); wz = warp_sum(wz); wzn = warp_sum(wzn);
    const float inv = 1.f / (acc + kEps);
    const float depth = wz / (acc + kEps), depth_ndc = wzn / (acc + kEps);
    float gd = a.g_depth ? a.g_depth[r] : 0.f;
    if (LOSS) {
        if (L.target_rgb) {
            float cr = 0.f, cg = 0.f, cb = 0.f;
#pragma unroll
            for (int k = 0; k < R; ++k) {
                if (i0 + k < c.s) {
                    const float w = al[k] * T[k];
                    cr += w * c0[k];
                    cg += w * c1[k];
                    cb += w * c2[k];
                }
            }
            cr = warp_sum(cr); cg = warp_sum(cg); cb = warp_sum(cb);
            if (white_for(a, r)) {
                cr = cr + (1.f - acc);
                cg = cg + (1.f - acc);
                cb = cb + (1.f - acc);
            }
            const float s2 = 2.f * L.rgb_scale;
            g0 += s2 * (cr - L.target_rgb[3 * r]);
            g1 += s2 * (cg - L.target_rgb[3 * r + 1]);
            g2 += s2 * (cb - L.target_rgb[3 * r + 2]);
        }
        if (depth_term(L, r)) {
            const float e = depth - L.target_depth[r];
            gd += L.depth_squared ? 2.f * L.depth_scale * e
                                  : L.depth_scale * (e > 0.f ? 1.f : (e < 0.f ? -1.f : 0.f));
        }
        if (mc_term(L, r)) {
            float w[R];
#pragma unroll
            for (int k = 0; k < R; ++k) w[k] = i0 + k < c.s ? al[k] * T[k] : 0.f;
            for (int b = 0; b < L.bins.nb; ++b) {
                const float x = bin_sum_blk<R>(w, L.bins, b, lane) + 1e-3f;
                const float gb = -(logf(x) + 1.f) * L.mc_scale;
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    const int i = i0 + k;
                    if (i >= L.bins.start[b] && i < L.bins.start[b + 1]) G[k] += gb;
                }
            }
        }
    }
    if (white_for(a, r)) gacc -= g0 + g1 + g2;
    const float gv = a.g_depth_var ? a.g_depth_var[r] : 0.f;
    const float gdn = (c.ndc && a.g_depth_ndc) ? a.g_depth_ndc[r] : 0.f;
    const float gvn = (c.ndc && a.g_depth_var_ndc) ? a.g_depth_var_ndc[r] : 0.f;
    float bsum = 0.f, bsum_n = 0.f;
    if (gv != 0.f || gvn != 0.f) {
#pragma unroll
        for (int k = 0; k < R; ++k) {
            if (i0 + k < c.s) {
                const float w = al[k] * T[k];
                const float zm = c.ndc ? depth_from_ndc(zz[k], c.oz, c.dz) : zz[k];
                bsum += w * (zm - depth);
                if (c.ndc) bsum_n += w * (zz[k] - depth_ndc);
            }
        }
        bsum = warp_sum(bsum);
        bsum_n = warp_sum(bsum_n);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const float zm = c.ndc ? depth_from_ndc(zz[k], c.oz, c.dz) : zz[k];
        float g = c0[k] * g0 + c1[k] * g1 + c2[k] * g2 + gacc + G[k];
        const float d = zm - depth;
        g += gd * d * inv + gv * (d * d - 2.f * bsum * d * inv);
        if (c.ndc) {
            const float dn = zz[k] - depth_ndc;
            g += gdn * dn * inv + gvn * (dn * dn - 2.f * bsum_n * dn * inv);
        }
        G[k] = g;
    }
    __syncwarp();   // every lane has read its stage rows before the gradients overwrite them
    if (exp_prefix) {
        // dL/dy_k = G_k e^{-y_k} T_k - sum_{i>k} G_i w_i: suffix sums in the lane, then
        // over the later lanes
        float after[R], run = 0.f;
#pragma unroll
        for (int k = R - 1; k >= 0; --k) {
            after[k] = run;
            if (i0 + k < c.s) run += G[k] * (al[k] * T[k]);
        }
        float inc = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float t = __shfl_down_sync(0xffffffffu, inc, o);
            if (lane + o < 32) inc += t;
        }
        float post = __shfl_down_sync(0xffffffffu, inc, 1);
        if (lane == 31) post = 0.f;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            const int i = i0 + k;
            if (i < c.s) {
                const float w = al[k] * T[k];
                const float dy = G[k] * ex_[k] * T[k] - (post + after[k]);
                dsig_out[i] = dy * c.ds * dl[k];
                if (drgb_out) {
                    drgb_out[3 * i] = w * g0;
                    drgb_out[3 * i + 1] = w * g1;
                    drgb_out[3 * i + 2] = w * g2;
                }
            }
        }
        return;
    }
    // reverse affine scan R_i = G_{i+1} a_{i+1} + p_{i+1} R_{i+1}, R_{S-1} = 0: sample
    // i's map x -> A_i + B_i x; a lane composes its block's maps, a suffix scan over
    // the lanes gives each block the R after it, and the lane then walks back.
    float ga[R], pp[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const bool in = i0 + k < c.s;
        ga[k] = in ? G[k] * al[k] : 0.f;
        pp[k] = in ? 1.f - al[k] + 1e-10f : 1.f;
    }
    const float ga_n = __shfl_down_sync(0xffffffffu, ga[0], 1);   // the next lane's first sample
    const float p_n = __shfl_down_sync(0xffffffffu, pp[0], 1);
    float A[R], B[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int i = i0 + k;
        const bool has_next = i < c.s && i + 1 < c.s;
        A[k] = has_next ? (k + 1 < R ? ga[k + 1] : ga_n) : 0.f;
        B[k] = has_next ? (k + 1 < R ? pp[k + 1] : p_n) : 0.f;
    }
    float FA = 0.f, FB = 1.f;   // this block's composed map
#pragma unroll
    for (int k = R - 1; k >= 0; --k) {
        FA = A[k] + B[k] * FA;
        FB = B[k] * FB;
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float A2 = __shfl_down_sync(0xffffffffu, FA, o);
        const float B2 = __shfl_down_sync(0xffffffffu, FB, o);
        if (lane + o < 32) {
            FA = FA + FB * A2;
            FB = FB * B2;
        }
    }
    float Rv = __shfl_down_sync(0xffffffffu, FA, 1);   // R of the first sample after this block
    if (lane == 31) Rv = 0.f;
#pragma unroll
    for (int k = R - 1; k >= 0; --k) {
        Rv = A[k] + B[k] * Rv;
        const int i = i0 + k;
        if (i < c.s) {
            const float dalpha = T[k] * (G[k] - Rv);
            float dx = -dalpha * ex_[k];
            dx = dx * c.ds;
            dsig_out[i] = -dx * dl[k];
            if (drgb_out) {
                const float w = al[k] * T[k];
                drgb_out[3 * i] = w * g0;
                drgb_out[3 * i + 1] = w * g1;
                drgb_out[3 * i + 2] = w * g2;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Staged variants: persistent warps, each owning rays r, r + W, r + 2W, ...
// (W warps in the grid).  Lane 0 of a warp copies the next ray's sigma, z and
// rgb (contiguous per ray) into the warp's other shared-memory stage with bulk
// asynchronous copies (cp.async.bulk, completion counted on an mbarrier) while
// the warp composites the current ray from shared memory (the blocked bodies
// above), so every warp keeps one ray's bytes in flight independently of its
// registers; the ray's per-sample outputs leave the stage by bulk copies too.
// Needs S % 4 == 0 and 16-byte aligned per-sample inputs and outputs (the bulk
// copies move 16-byte multiples).  A wait that runs out (4 s) raises the device
// flag and ends the warp.
// ---------------------------------------------------------------------------

constexpr int kStagedWarps = 8;
constexpr int kStages = 2;   // rays per warp in shared memory: one composited, the rest in flight

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     tc::smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(tc::smem_u32(bar))
                 : "memory");
}

// Shared -> global bulk copy (bulk async group of the issuing thread).
__device__ __forceinline__ void bulk_s2g(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(tc::smem_u32(src)),
                 "r"(bytes)
                 : "memory");
}

// Stage layout per warp and stage: sigma[S] | z[S] | rgb[3 S] (floats).
__host__ __device__ __forceinline__ int staged_floats(int s) { return 5 * s; }

__device__ __forceinline__ void stage_ray(const srf_composite_args& a, int r, float* st, uint64_t* bar) {
    const int s = a.n_samples;
    const uint32_t b1 = uint32_t(s) * 4u;
    const uint32_t bytes = a.rgb ? 5u * b1 : 2u * b1;
    tc::mbar_arrive_expect_tx(bar, bytes);
    bulk_g2s(st, a.sigma + int64_t(r) * s, b1, bar);
    bulk_g2s(st + s, a.z + int64_t(r) * s, b1, bar);
    if (a.rgb) bulk_g2s(st + 2 * s, a.rgb + int64_t(r) * s * 3, 3u * b1, bar);
}

template <int R, bool LOSS, bool BWD>
__global__ void __launch_bounds__(kStagedWarps * 32, 3) composite_staged_kernel(srf_composite_args a, LossArgs L,
                                                                                 int* flag) {
    extern __shared__ __align__(128) float smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int s = a.n_samples;
    float* mine = smem + size_t(warp) * kStages * staged_floats(s);
    uint64_t* bars =
        reinterpret_cast<uint64_t*>(smem + size_t(kStagedWarps) * kStages * staged_floats(s)) + kStages * warp;
    const int stride = gridDim.x * kStagedWarps;
    const int r0 = blockIdx.x * kStagedWarps + warp;
    if (lane == 0) {
        for (int i = 0; i < kStages; ++i) tc::mbar_init(&bars[i], 1);
        tc::fence_barrier_init();
    }
    __syncwarp();
    // the first kStages - 1 rays go out before the loop; iteration k prefetches ray
    // k + kStages - 1 into the stage that ray k - 1 used
    if (lane == 0)
        for (int i = 0; i + 1 < kStages; ++i)
            if (r0 + i * stride < a.n_rays) stage_ray(a, r0 + i * stride, mine + i * staged_floats(s), &bars[i]);
    uint32_t phases = 0u;   // bit i: the mbarrier phase stage i waits for next
    int k = 0;
    for (int r = r0; r < a.n_rays; ++k, r += stride) {
        const int cur = k % kStages;
        float* st = mine + cur * staged_floats(s);
        const int ahead = r + (kStages - 1) * stride;
        if (ahead < a.n_rays && lane == 0) {
            const int nxt = (k + kStages - 1) % kStages;
            tc::bulk_wait_read_all();   // the bulk stores of ray k - 1 have read that stage
            stage_ray(a, ahead, mine + nxt * staged_floats(s), &bars[nxt]);
        }
        if (!tc::mbar_wait(&bars[cur], (phases >> cur) & 1u, nullptr)) {
            raise_flag(flag, kFlagTimeout);
            // drain (bounded) whatever is still in flight into this warp's stages
            for (int i = 1; i < kStages; ++i) {
                const int st2 = (k + i) % kStages;
                if (r + i * stride < a.n_rays) tc::mbar_wait(&bars[st2], (phases >> st2) & 1u, nullptr);
            }
            if (lane == 0) tc::bulk_wait_all();
            return;
        }
        phases ^= 1u << cur;
        RayCtx c = make_ctx(a, r);
        c.sigma = st;
        c.z = st + s;
        const float* rgb = a.rgb ? st + 2 * s : nullptr;
        const int64_t ro = int64_t(r) * s;
        // the per-sample outputs land in this stage (weights / d_sigma over sigma,
        // d_rgb over rgb) and leave by bulk copies
        if (BWD)
            bwd_ray_blk<R, LOSS>(a, L, r, c, rgb, st, a.d_rgb ? st + 2 * s : nullptr);
        else
            fwd_ray_blk<R, LOSS>(a, L, r, c, rgb, st);
        tc::fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) {
            if (BWD) {
                bulk_s2g(a.d_sigma + ro, st, uint32_t(s) * 4u);
                if (a.d_rgb) bulk_s2g(a.d_rgb + ro * 3, st + 2 * s, uint32_t(s) * 12u);
            } else if (a.weights) {
                bulk_s2g(a.weights + ro, st, uint32_t(s) * 4u);
            }
            tc::bulk_commit_group();
        }
        __syncwarp();
    }
    if (lane == 0) tc::bulk_wait_all();
}

// out[r, c] = sum_s w[r, s] x[r, s, c] (one warp per ray); the adjoint gives
// dw[r, s] = sum_c g[r, c] x[r, s, c] and dx[r, s, c] = w[r, s] g[r, c].
__global__ void weighted_sum_kernel(const float* __restrict__ w, const float* __restrict__ x, int n, int s, int c,
                                    float* out) {
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int r = blockIdx.x * (blockDim.x >> 5) + warp;
    if (r >= n) return;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int i = lane; i < s; i += 32) {
        float wi = w[int64_t(r) * s + i];
        for (int k = 0; k < c; ++k) acc[k] += wi * x[(int64_t(r) * s + i) * c + k];
    }
    for (int k = 0; k < c; ++k) {
        float v = warp_sum(acc[k]);
        if (lane == 0) out[int64_t(r) * c + k] = v;
    }
}

__global__ void weighted_sum_bwd_kernel(const float* __restrict__ w, const float* __restrict__ x,
                                        const float* __restrict__ g, int n, int s, int c, float* dw, float* dx) {
    int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= int64_t(n) * s) return;
    int64_t r = idx / s;
    float acc = 0.f;
    for (int k = 0; k < c; ++k) {
        float gk = g[r * c + k];
        acc += gk * x[idx * c + k];
        if (dx) dx[idx * c + k] = w[idx] * gk;
    }
    if (dw) dw[idx] = acc;
}

int check_args(const srf_composite_args* a, bool bwd) {
    if (!a || !a->sigma || !a->z || !a->rays_d) return SRF_ERR_NULL;
    if ((a->flags & SRF_COMPOSITE_NDC) && (!a->rays_o || !a->rays_d_ndc)) return SRF_ERR_NULL;
    if (a->n_rays < 0 || a->n_samples < 1 || a->n_samples > 16384) return SRF_ERR_SHAPE;
    if (bwd && !a->d_sigma) return SRF_ERR_NULL;
    return SRF_OK;
}

template <class K>
int launch(K kernel, const srf_composite_args* a, void* stream) {
    size_t per_warp = size_t(2) * a->n_samples * sizeof(float);
    int warps = int(49152 / per_warp);
    if (warps > 8) warps = 8;
    if (warps < 1) warps = 1;
    size_t smem = per_warp * warps;
    if (smem > 49152) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) {
            set_cuda_error(e);
            return SRF_ERR_CUDA;
        }
    }
    kernel<<<grid_1d(a->n_rays, warps), warps * 32, smem, as_stream(stream)>>>(*a);
    return launch_status();
}

// Rounds of 32 samples of the register-resident kernels for rays of n samples
// (rounded up to an even count, <= 8), or 0 for the shared-memory kernels.
inline int reg_rounds(int n) {
    int r = (n + 31) / 32;
    r += r & 1;
    return r <= 8 ? r : 0;
}

template <class K>
int launch_reg(K kernel, const srf_composite_args* a, const LossArgs& L, void* stream) {
    kernel<<<grid_1d(a->n_rays, 8), 256, 0, as_stream(stream)>>>(*a, L);
    return launch_status();
}

bool stageable(const srf_composite_args* a) {
    auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; };
    return (a->n_samples & 3) == 0 && al16(a->sigma) && al16(a->z) && (!a->rgb || al16(a->rgb)) &&
           (!a->weights || al16(a->weights)) && (!a->d_sigma || al16(a->d_sigma)) && (!a->d_rgb || al16(a->d_rgb));
}

template <int R, bool LOSS, bool BWD>
int launch_staged(const srf_composite_args* a, const LossArgs& L, void* stream) {
    auto kernel = composite_staged_kernel<R, LOSS, BWD>;
    const size_t smem = size_t(kStagedWarps) * kStages * staged_floats(a->n_samples) * sizeof(float) +
                        size_t(kStagedWarps) * kStages * sizeof(uint64_t);
    static int configured = 0;   // per instantiation: the largest shared-memory size set so far
    if (int(smem) > configured) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) {
            set_cuda_error(e);
            return SRF_ERR_CUDA;
        }
        configured = int(smem);
    }
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kStagedWarps * 32, smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return SRF_ERR_CUDA;
    }
    const int64_t need = (int64_t(a->n_rays) + kStagedWarps - 1) / kStagedWarps;
    const int blocks = int(need < int64_t(sms) * per_sm ? need : int64_t(sms) * per_sm);
    kernel<<<blocks, kStagedWarps * 32, smem, as_stream(stream)>>>(*a, L, device_flag());
    return launch_status();
}

template <bool LOSS>
int forward_reg(const srf_composite_args* a, const LossArgs& L, void* stream) {
    const bool staged = stageable(a);
    switch (reg_rounds(a->n_samples)) {
        case 2: return staged ? launch_staged<2, LOSS, false>(a, L, stream)
                              : launch_reg(composite_fwd_reg_kernel<2, LOSS>, a, L, stream);
        case 4: return staged ? launch_staged<4, LOSS, false>(a, L, stream)
                              : launch_reg(composite_fwd_reg_kernel<4, LOSS>, a, L, stream);
        case 6: return staged ? launch_staged<6, LOSS, false>(a, L, stream)
                              : launch_reg(composite_fwd_reg_kernel<6, LOSS>, a, L, stream);
        case 8: return staged ? launch_staged<8, LOSS, false>(a, L, stream)
                              : launch_reg(composite_fwd_reg_kernel<8, LOSS>, a, L, stream);
        default: return SRF_ERR_UNSUPPORTED;
    }
}

template <bool LOSS>
int backward_reg(const srf_composite_args* a, const LossArgs& L, void* stream) {
    const bool staged = stageable(a);
    switch (reg_rounds(a->n_samples)) {
        case 2: return staged ? launch_staged<2, LOSS, true>(a, L, stream)
                              : launch_reg(composite_bwd_reg_kernel<2, LOSS>, a, L, stream);
        case 4: return staged ? launch_staged<4, LOSS, true>(a, L, stream)
                              : launch_reg(composite_bwd_reg_kernel<4, LOSS>, a, L, stream);
        case 6: return staged ? launch_staged<6, LOSS, true>(a, L, stream)
                              : launch_reg(composite_bwd_reg_kernel<6, LOSS>, a, L, stream);
        case 8: return staged ? launch_staged<8, LOSS, true>(a, L, stream)
                              : launch_reg(composite_bwd_reg_kernel<8, LOSS>, a, L, stream);
        default: return SRF_ERR_UNSUPPORTED;
    }
}

int make_loss(const srf_composite_args* a, const srf_composite_loss* l, LossArgs* L) {
    if (!l || !l->loss) return SRF_ERR_NULL;
    if (l->n_depth_rays < 0 || l->n_mc_rays < 0 || l->num_bins < 0 || l->num_bins > 32) return SRF_ERR_SHAPE;
    *L = LossArgs{};
    L->loss = l->loss;
    L->target_rgb = l->target_rgb;
    L->rgb_scale = a->n_rays > 0 ? l->rgb_weight / float(3 * a->n_rays) : 0.f;
    if (l->target_depth && l->n_depth_rays > 0) {
        L->target_depth = l->target_depth;
        L->depth_mask = l->depth_mask;
        L->depth_scale = l->depth_weight / float(l->n_depth_rays);
        L->depth_squared = l->depth_squared != 0;
    }
    if (l->num_bins > 0 && l->n_mc_rays > 0) {
        if (!bin_layout(a->n_samples, l->num_bins, &L->bins)) return SRF_ERR_SHAPE;
        L->mc_mask = l->mc_mask;
        L->mc_scale = l->mc_weight / float(l->n_mc_rays);
    } else {
        L->bins.nb = 0;
    }
    return SRF_OK;
}

}  // namespace
}  // namespace srf

using namespace srf;

extern "C" int srf_composite_forward(const srf_composite_args* args, void* stream) {
    int st = check_args(args, false);
    if (st != SRF_OK || args->n_rays == 0) return st;
    if ((args->flags & SRF_COMPOSITE_EXP_PREFIX) && !reg_rounds(args->n_samples)) return SRF_ERR_UNSUPPORTED;
    if (reg_rounds(args->n_samples)) return forward_reg<false>(args, LossArgs{}, stream);
    return launch(composite_fwd_kernel, args, stream);
}

extern "C" int srf_composite_backward(const srf_composite_args* args, void* stream) {
    int st = check_args(args, true);
    if (st != SRF_OK || args->n_rays == 0) return st;
    if ((args->flags & SRF_COMPOSITE_EXP_PREFIX) && !reg_rounds(args->n_samples)) return SRF_ERR_UNSUPPORTED;
    if (reg_rounds(args->n_samples)) return backward_reg<false>(args, LossArgs{}, stream);
    return launch(composite_bwd_kernel, args, stream);
}

extern "C" int srf_composite_forward_loss(const srf_composite_args* args, const srf_composite_loss* loss,
                                          void* stream) {
    int st = check_args(args, false);
    if (st != SRF_OK) return st;
    LossArgs L;
    if ((st = make_loss(args, loss, &L)) != SRF_OK || args->n_rays == 0) return st;
    if (!reg_rounds(args->n_samples)) return SRF_ERR_UNSUPPORTED;
    return forward_reg<true>(args, L, stream);
}

extern "C" int srf_composite_backward_loss(const srf_composite_args* args, const srf_composite_loss* loss,
                                           void* stream) {
    int st = check_args(args, true);
    if (st != SRF_OK) return st;
    LossArgs L;
    if ((st = make_loss(args, loss, &L)) != SRF_OK || args->n_rays == 0) return st;
    if (!reg_rounds(args->n_samples)) return SRF_ERR_UNSUPPORTED;
    return backward_reg<true>(args, L, stream);
}

extern "C" int srf_weighted_sum(const float* weights, const float* values, int n_rays, int n_samples, int channels,
                                float* out, void* stream) {
    if (!weights || !values || !out) return SRF_ERR_NULL;
    if (n_rays < 0 || n_samples < 1 || channels < 1 || channels > 4) return SRF_ERR_SHAPE;
    if (n_rays == 0) return SRF_OK;
    weighted_sum_kernel<<<grid_1d(n_rays, 8), 256, 0, as_stream(stream)>>>(weights, values, n_rays, n_samples,
                                                                          channels, out);
    return launch_status();
}

extern "C" int srf_weighted_sum_backward(const float* weights, const float* values, const float* g_out, int n_rays,
                                         int n_samples, int channels, float* d_weights, float* d_values,
                                         void* stream) {
    if (!weights || !values || !g_out) return SRF_ERR_NULL;
    if (n_rays < 0 || n_samples < 1 || channels < 1 || channels > 4) return SRF_ERR_SHAPE;
    if (n_rays == 0) return SRF_OK;
    int64_t tot = int64_t(n_rays) * n_samples;
    weighted_sum_bwd_kernel<<<grid_1d(tot, 256), 256, 0, as_stream(stream)>>>(weights, values, g_out, n_rays,
                                                                             n_samples, channels, d_weights,
                                                                             d_values);
    return launch_status();
}
