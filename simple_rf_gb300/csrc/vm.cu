// TensoRF VM (vector-matrix) plane/line lookups, alpha-mask query, sample
// masks and stream compaction (SimpleTensoRF09.py:701-765, 1214-1272, 1342-1349).
//
// Planes and lines are stored channels-last (plane (H,W,R), line (L,R)) so one
// bilinear corner is R contiguous floats: a corner of a 16-component plane is a
// single 64-byte line, read with 128-bit loads.  One thread handles one
// (point, plane) pair for the density path, and one point for colour.
#include <mutex>
#include <type_traits>

#include "autotune.cuh"
#include "srf_common.cuh"

namespace srf {
namespace {

__constant__ int kMatrixAxes[3][2] = {{0, 1}, {0, 2}, {1, 2}};   // SimpleTensoRF09.py:1131
__constant__ int kVectorAxes[3] = {2, 1, 0};                      // SimpleTensoRF09.py:1132
constexpr int kMatrixAxesHost[3][2] = {{0, 1}, {0, 2}, {1, 2}};   // the same axes for host code
constexpr int kVectorAxesHost[3] = {2, 1, 0};

// Bilinear taps of torch's CPU grid sampler (align_corners=True, zeros padding):
// ix = (x + 1) * ((W - 1) / 2); weights from the fractional parts.
struct Taps {
    int idx[4];    // flat corner index (y * W + x), -1 when out of bounds
    float w[4];
};

__device__ __forceinline__ Taps bilinear(float gx, float gy, int h, int w) {
    Taps t;
    float ix = (gx + 1.f) * (float(w - 1) * 0.5f);
    float iy = (gy + 1.f) * (float(h - 1) * 0.5f);
    // far-outside coordinates only ever touch padding; clamp before the int
    // conversion so the corner indices stay small
    if (isfinite(ix)) ix = fminf(fmaxf(ix, -4.f), float(w) + 4.f);
    if (isfinite(iy)) iy = fminf(fmaxf(iy, -4.f), float(h) + 4.f);
    float x0f = floorf(ix), y0f = floorf(iy);
    float fw = ix - x0f, fe = 1.f - fw;
    float fn = iy - y0f, fs = 1.f - fn;
    int x0 = int(x0f), y0 = int(y0f);
    const int dx[4] = {0, 1, 0, 1}, dy[4] = {0, 0, 1, 1};
    const float ww[4] = {fs * fe, fs * fw, fn * fe, fn * fw};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        int xi = x0 + dx[c], yi = y0 + dy[c];
        bool ok = xi >= 0 && xi < w && yi >= 0 && yi < h && isfinite(ix) && isfinite(iy);
        t.idx[c] = ok ? yi * w + xi : -1;
        t.w[c] = ok ? ww[c] : 0.f;
    }
    return t;
}

// Line lookup: grid (0, v) on a (L, 1) image; x taps collapse to ix = 0.
__device__ __forceinline__ Taps line_taps(float gv, int len) {
    return bilinear(0.f, gv, len, 1);
}

// sum_r plane[r] * line[r] for R components (R multiple of 4 uses float4 loads).
__device__ __forceinline__ float vm_dot(const float* __restrict__ plane, const float* __restrict__ line, int R,
                                        const Taps& pt, const Taps& lt) {
    float acc = 0.f;
    if ((R & 3) == 0) {
        for (int r = 0; r < R; r += 4) {
            float4 pv = make_float4(0.f, 0.f, 0.f, 0.f), lv = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (pt.idx[c] >= 0) {
                    float4 v = *reinterpret_cast<const float4*>(plane + int64_t(pt.idx[c]) * R + r);
                    pv.x += v.x * pt.w[c]; pv.y += v.y * pt.w[c]; pv.z += v.z * pt.w[c]; pv.w += v.w * pt.w[c];
                }
                if (lt.idx[c] >= 0) {
                    float4 v = *reinterpret_cast<const float4*>(line + int64_t(lt.idx[c]) * R + r);
                    lv.x += v.x * lt.w[c]; lv.y += v.y * lt.w[c]; lv.z += v.z * lt.w[c]; lv.w += v.w * lt.w[c];
                }
            }
            acc += pv.x * lv.x;
            acc += pv.y * lv.y;
            acc += pv.z * lv.z;
            acc += pv.w * lv.w;
        }
    } else {
        for (int r = 0; r < R; ++r) {
            float pv = 0.f, lv = 0.f;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (pt.idx[c] >= 0) pv += plane[int64_t(pt.idx[c]) * R + r] * pt.w[c];
                if (lt.idx[c] >= 0) lv += line[int64_t(lt.idx[c]) * R + r] * lt.w[c];
            }
            acc += pv * lv;
        }
    }
    return acc;
}

__device__ __forceinline__ void plane_taps(const srf_vm_grid& g, int i, const float* p, Taps& pt, Taps& lt) {
    int m0 = kMatrixAxes[i][0], m1 = kMatrixAxes[i][1], v = kVectorAxes[i];
    pt = bilinear(p[m0], p[m1], g.res[m1], g.res[m0]);
    lt = line_taps(p[v], g.res[v]);
}

__global__ void density_fwd_kernel(srf_vm_grid g, const float* __restrict__ pts, int64_t n, float* out) {
    int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float* q = pts + 3 * p;
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        Taps pt, lt;
        plane_taps(g, i, q, pt, lt);
        acc = acc + vm_dot(g.planes[i], g.lines[i], g.n_comp[i], pt, lt);
    }
    out[p] = acc;
}

// 4 consecutive floats (16-byte aligned) of one corner: a plane's or a line's R components
// are contiguous in the channels-last layout.
__device__ __forceinline__ float4 corner4(const float* __restrict__ base, int idx, int R, int r) {
    return *reinterpret_cast<const float4*>(base + int64_t(idx) * R + r);
}

__device__ __forceinline__ void red_add4(float* dst, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst), "f"(a), "f"(b), "f"(c), "f"(d)
                 : "memory");
}

// Bilinearly interpolated components r..r+3 of a plane and of a line.
__device__ __forceinline__ void interp4(const float* __restrict__ pl, const float* __restrict__ ln, int R, int r,
                                        const Taps& pt, const Taps& lt, float4& pv, float4& lv) {
    pv = make_float4(0.f, 0.f, 0.f, 0.f);
    lv = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        if (pt.idx[c] >= 0) {
            float4 v = corner4(pl, pt.idx[c], R, r);
            float w = pt.w[c];
            pv.x += v.x * w; pv.y += v.y * w; pv.z += v.z * w; pv.w += v.w * w;
        }
        if (lt.idx[c] >= 0) {
            float4 v = corner4(ln, lt.idx[c], R, r);
            float w = lt.w[c];
            lv.x += v.x * w; lv.y += v.y * w; lv.z += v.z * w; lv.w += v.w * w;
        }
    }
}

// Components are grouped by 4 (R multiple of 4, checked on the host) so each
// corner access is one 128-bit load.
__global__ void color_fwd_kernel(srf_vm_grid g, const float* __restrict__ pts, int64_t n, int ld, float* out) {
    int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float* q = pts + 3 * p;
    float* o = out + p * ld;
    int off = 0;
    for (int i = 0; i < 3; ++i) {
        Taps pt, lt;
        plane_taps(g, i, q, pt, lt);
        const int R = g.n_comp[i];
        const float* pl = g.planes[i];
        const float* ln = g.lines[i];
        if ((R & 3) == 0) {
            for (int r = 0; r < R; r += 4) {
                float4 pv, lv;
                interp4(pl, ln, R, r, pt, lt, pv, lv);
                o[off + r] = pv.x * lv.x;
                o[off + r + 1] = pv.y * lv.y;
                o[off + r + 2] = pv.z * lv.z;
                o[off + r + 3] = pv.w * lv.w;
            }
        } else {
            for (int r = 0; r < R; ++r) {
                float pv = 0.f, lv = 0.f;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    if (pt.idx[c] >= 0) pv += pl[int64_t(pt.idx[c]) * R + r] * pt.w[c];
                    if (lt.idx[c] >= 0) lv += ln[int64_t(lt.idx[c]) * R + r] * lt.w[c];
                }
                o[off + r] = pv * lv;
            }
        }
        off += R;
    }
}

// Adjoint: d plane[r] at corner c += w_c * d_r * line_value[r] (and symmetrically),
// four components per 128-bit reduction.  Colour: d_features (P, ld) per component;
// density: one scalar per point.
__global__ void vm_bwd_kernel(srf_vm_grid gg, srf_vm_grid g, const float* __restrict__ pts, int64_t n,
                              const float* __restrict__ dfeat, int ld, int per_component) {
    int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float* q = pts + 3 * p;
    const float ds = per_component ? 0.f : dfeat[p];
    if (!per_component && ds == 0.f) return;
    int off = 0;
    for (int i = 0; i < 3; ++i) {
        Taps pt, lt;
        plane_taps(g, i, q, pt, lt);
        const int R = g.n_comp[i];
        float* gpl = gg.planes[i];
        float* gln = gg.lines[i];
        if ((R & 3) != 0 || (per_component && ((ld | off) & 3) != 0)) {
            // component counts that are not multiples of 4: scalar loads and atomics
            const float* pl = g.planes[i];
            const float* ln = g.lines[i];
            for (int r = 0; r < R; ++r) {
                float pv = 0.f, lv = 0.f;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    if (pt.idx[c] >= 0) pv += pl[int64_t(pt.idx[c]) * R + r] * pt.w[c];
                    if (lt.idx[c] >= 0) lv += ln[int64_t(lt.idx[c]) * R + r] * lt.w[c];
                }
                float d = per_component ? dfeat[p * ld + off + r] : ds;
                float dp = d * lv, dl = d * pv;
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    if (pt.idx[c] >= 0 && dp != 0.f) atomicAdd(gpl + int64_t(pt.idx[c]) * R + r, dp * pt.w[c]);
                    if (lt.idx[c] >= 0 && dl != 0.f) atomicAdd(gln + int64_t(lt.idx[c]) * R + r, dl * lt.w[c]);
                }
            }
            off += R;
            continue;
        }
        for (int r = 0; r < R; r += 4) {
            float4 d = per_component ? *reinterpret_cast<const float4*>(dfeat + p * ld + off + r)
                                     : make_float4(ds, ds, ds, ds);
            if (d.x == 0.f && d.y == 0.f && d.z == 0.f && d.w == 0.f) continue;
            float4 pv, lv;
            interp4(g.planes[i], g.lines[i], R, r, pt, lt, pv, lv);
            const float4 dp = make_float4(d.x * lv.x, d.y * lv.y, d.z * lv.z, d.w * lv.w);
            const float4 dl = make_float4(d.x * pv.x, d.y * pv.y, d.z * pv.z, d.w * pv.w);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (pt.idx[c] >= 0) {
                    const float w = pt.w[c];
                    red_add4(gpl + int64_t(pt.idx[c]) * R + r, dp.x * w, dp.y * w, dp.z * w, dp.w * w);
                }
                if (lt.idx[c] >= 0) {
                    const float w = lt.w[c];
                    red_add4(gln + int64_t(lt.idx[c]) * R + r, dl.x * w, dl.y * w, dl.z * w, dl.w * w);
                }
            }
        }
        off += R;
    }
}

// Group forms of the colour gather and of the scatter-add adjoint: G lanes share a
// point and lane j of the group takes components 4j, 4j + 4G, ... of every plane,
// so each corner access of a warp covers whole contiguous rows of components
// (192 bytes for R = 48) instead of 32 unrelated 16-byte pieces.  Needs every
// R_i and the feature row length to be multiples of 4 (checked on the host).
template <int G>
__global__ void color_fwd_group_kernel(srf_vm_grid g, const float* __restrict__ pts, int64_t n, int ld,
                                       float* __restrict__ out) {
    const int j = threadIdx.x % G;
    const int64_t p = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) / G;
    if (p >= n) return;
    const float* q = pts + 3 * p;
    float* o = out + p * ld;
    int off = 0;
    for (int i = 0; i < 3; ++i) {
        Taps pt, lt;
        plane_taps(g, i, q, pt, lt);
        const int R = g.n_comp[i];
#pragma unroll 4
        for (int r = 4 * j; r < R; r += 4 * G) {
            float4 pv, lv;
            interp4(g.planes[i], g.lines[i], R, r, pt, lt, pv, lv);
            *reinterpret_cast<float4*>(o + off + r) = make_float4(pv.x * lv.x, pv.y * lv.y, pv.z * lv.z, pv.w * lv.w);
        }
        off += R;
    }
}

template <int G>
__global__ void vm_bwd_group_kernel(srf_vm_grid gg, srf_vm_grid g, const float* __restrict__ pts, int64_t n,
                                    const float* __restrict__ dfeat, int ld, int per_component) {
    const int j = threadIdx.x % G;
    const int64_t p = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) / G;
    if (p >= n) return;
    const float* q = pts + 3 * p;
    const float ds = per_component ? 0.f : dfeat[p];
    if (!per_component && ds == 0.f) return;
    int off = 0;
    for (int i = 0; i < 3; ++i) {
        Taps pt, lt;
        plane_taps(g, i, q, pt, lt);
        const int R = g.n_comp[i];
        float* gpl = gg.planes[i];
        float* gln = gg.lines[i];
#pragma unroll 4
        for (int r = 4 * j; r < R; r += 4 * G) {
            const float4 d = per_component ? *reinterpret_cast<const float4*>(dfeat + p * ld + off + r)
                                           : make_float4(ds, ds, ds, ds);
            if (d.x == 0.f && d.y == 0.f && d.z == 0.f && d.w == 0.f) continue;
            float4 pv, lv;
            interp4(g.planes[i], g.lines[i], R, r, pt, lt, pv, lv);
            const float4 dp = make_float4(d.x * lv.x, d.y * lv.y, d.z * lv.z, d.w * lv.w);
            const float4 dl = make_float4(d.x * pv.x, d.y * pv.y, d.z * pv.z, d.w * pv.w);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (pt.idx[c] >= 0) {
                    const float w = pt.w[c];
                    red_add4(gpl + int64_t(pt.idx[c]) * R + r, dp.x * w, dp.y * w, dp.z * w, dp.w * w);
                }
                if (lt.idx[c] >= 0) {
                    const float w = lt.w[c];
                    red_add4(gln + int64_t(lt.idx[c]) * R + r, dl.x * w, dl.y * w, dl.z * w, dl.w * w);
                }
            }
        }
        off += R;
    }
}

// Lanes per point for the group kernels: the largest power of two (at most 16) that
// divides every R_i / 4, so every lane of a group takes the same number of
// four-component pieces (R = 48: 4 lanes x 3 pieces, each lane's loads independent
// of one another); 0 when some R_i is not a multiple of 4 (per-thread kernels).
int group_lanes(const srf_vm_grid& g) {
    int G = 16;
    for (int i = 0; i < 3; ++i) {
        if (g.n_comp[i] & 3) return 0;
        while (G > 1 && (g.n_comp[i] / 4) % G) G >>= 1;
    }
    return G;
}

template <class F>
int launch_grouped(int G, int64_t n, F&& launch) {
    switch (G) {
        case 1: return launch(std::integral_constant<int, 1>{});
        case 2: return launch(std::integral_constant<int, 2>{});
        case 4: return launch(std::integral_constant<int, 4>{});
        case 8: return launch(std::integral_constant<int, 8>{});
        case 16: return launch(std::integral_constant<int, 16>{});
        default: return launch(std::integral_constant<int, 32>{});
    }
}

// CP decomposition (CpDecomposedTensor, SimpleTensoRF09.py:964-1123): three lines,
// line i along world axis kVectorAxes[i], all with the same R components;
// density = sum_r prod_i line_i[r], colour features = prod_i line_i[r] per r.
__device__ __forceinline__ void cp_taps(const srf_vm_grid& g, const float* p, Taps (&t)[3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) t[i] = line_taps(p[kVectorAxes[i]], g.res[kVectorAxes[i]]);
}

__device__ __forceinline__ float line_value(const float* __restrict__ line, int R, int r, const Taps& t) {
    float v = 0.f;
#pragma unroll
    for (int c = 0; c < 4; ++c)
        if (t.idx[c] >= 0) v += line[int64_t(t.idx[c]) * R + r] * t.w[c];
    return v;
}

__global__ void cp_fwd_kernel(srf_vm_grid g, const float* __restrict__ pts, int64_t n, int per_component,
                              float* out) {
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= n) return;
    Taps t[3];
    cp_taps(g, pts + 3 * p, t);
    const int R = g.n_comp[0];
    float acc = 0.f;
    for (int r = 0; r < R; ++r) {
        const float v = line_value(g.lines[0], R, r, t[0]) * line_value(g.lines[1], R, r, t[1]) *
                        line_value(g.lines[2], R, r, t[2]);
        if (per_component) out[p * R + r] = v;
        else acc += v;
    }
    if (!per_component) out[p] = acc;
}

// d line_i[r] at its taps += w * d_r * prod_{j != i} line_j[r]
__global__ void cp_bwd_kernel(srf_vm_grid gg, srf_vm_grid g, const float* __restrict__ pts, int64_t n,
                              const float* __restrict__ dfeat, int per_component) {
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= n) return;
    Taps t[3];
    cp_taps(g, pts + 3 * p, t);
    const int R = g.n_comp[0];
    for (int r = 0; r < R; ++r) {
        const float d = per_component ? dfeat[p * R + r] : dfeat[p];
        if (d == 0.f) continue;
        const float v[3] = {line_value(g.lines[0], R, r, t[0]), line_value(g.lines[1], R, r, t[1]),
                            line_value(g.lines[2], R, r, t[2])};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float di = d * v[(i + 1) % 3] * v[(i + 2) % 3];
            if (di == 0.f) continue;
#pragma unroll
            for (int c = 0; c < 4; ++c)
                if (t[i].idx[c] >= 0) atomicAdd(gg.lines[i] + int64_t(t[i].idx[c]) * R + r, di * t[i].w[c]);
        }
    }
}

// AlphaGridMask.sample_alpha + "> 0": true iff an occupied in-bound corner has a
// positive trilinear weight (all terms are >= 0, so the float sum is positive
// exactly then).  Weights use torch's CPU 3-D formula ((x1 - ix) * (y1 - iy) * ...).
__device__ __forceinline__ bool alpha_positive(const float* __restrict__ vol, int d, int h, int w, float x, float y,
                                               float z) {
    float ix = ((x + 1.f) / 2.f) * float(w - 1);
    float iy = ((y + 1.f) / 2.f) * float(h - 1);
    float iz = ((z + 1.f) / 2.f) * float(d - 1);
    if (!(isfinite(ix) && isfinite(iy) && isfinite(iz))) return false;
    // outside [-1, size] every corner is padding
    if (ix < -1.f || iy < -1.f || iz < -1.f || ix > float(w) || iy > float(h) || iz > float(d)) return false;
    float x0 = floorf(ix), y0 = floorf(iy), z0 = floorf(iz);
    float x1 = x0 + 1.f, y1 = y0 + 1.f, z1 = z0 + 1.f;
    float wx[2] = {x1 - ix, ix - x0}, wy[2] = {y1 - iy, iy - y0}, wz[2] = {z1 - iz, iz - z0};
    int xi0 = int(x0), yi0 = int(y0), zi0 = int(z0);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        int cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
        int xi = xi0 + cx, yi = yi0 + cy, zi = zi0 + cz;
        if (xi < 0 || xi >= w || yi < 0 || yi >= h || zi < 0 || zi >= d) continue;
        float wt = wx[cx] * wy[cy] * wz[cz];
        if (wt > 0.f && vol[(int64_t(zi) * h + yi) * w + xi] * wt > 0.f) return true;
    }
    return false;
}

__global__ void alpha_query_kernel(const float* __restrict__ vol, int d, int h, int w, const float* __restrict__ p,
                                   int64_t n, uint8_t* out) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = alpha_positive(vol, d, h, w, p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}

struct Box {
    float lo[3], hi[3];
};

__global__ void sample_mask_kernel(const float* __restrict__ o, const float* __restrict__ dir,
                                   const float* __restrict__ z, int n, int s, Box box, const float* __restrict__ vol,
                                   int vd, int vh, int vw, Box abox, float* pn, uint8_t* mask) {
    int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= int64_t(n) * s) return;
    int r = int(idx / s);
    float zz = z[idx];
    float q[3];
    bool inside = true;
    // products and sums round separately, like the reference's torch ops
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        q[a] = __fadd_rn(o[3 * r + a], __fmul_rn(dir[3 * r + a], zz));   // SimpleTensoRF09.py:261
        inside = inside && box.lo[a] <= q[a] && q[a] <= box.hi[a];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
        pn[3 * idx + a] = __fsub_rn(__fmul_rn((q[a] - box.lo[a]) / (box.hi[a] - box.lo[a]), 2.f), 1.f);
    if (inside && vol) {
        float an[3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
            an[a] = __fsub_rn(__fmul_rn((q[a] - abox.lo[a]) / (abox.hi[a] - abox.lo[a]), 2.f), 1.f);
        inside = alpha_positive(vol, vd, vh, vw, an[0], an[1], an[2]);
    }
    mask[idx] = inside;
}

__global__ void threshold_kernel(const float* __restrict__ x, int64_t n, float thr, uint8_t* m) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) m[i] = x[i] > thr;
}

// ---- compaction: per-block counts -> exclusive scan of block counts -> write
constexpr int kCompactBlock = 1024;

__global__ void count_kernel(const uint8_t* __restrict__ mask, int64_t n, int* block_counts) {
    __shared__ int warp_counts[32];
    int64_t i = int64_t(blockIdx.x) * kCompactBlock + threadIdx.x;
    int v = i < n ? (mask[i] != 0) : 0;
    unsigned b = __ballot_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0) warp_counts[threadIdx.x >> 5] = __popc(b);
    __syncthreads();
    if (threadIdx.x < 32) {
        int c = warp_counts[threadIdx.x];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (threadIdx.x == 0) block_counts[blockIdx.x] = c;
    }
}

// Single-block exclusive scan over the block counts (in place), total -> *count.
__global__ void scan_counts_kernel(int* counts, int nb, int* total) {
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += blockDim.x) {
        int i = base + threadIdx.x;
        int v = i < nb ? counts[i] : 0;
        int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        int inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        __shared__ int wsum[32];
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            int ws = lane < int(blockDim.x >> 5) ? wsum[lane] : 0;
            int wi = ws;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += t;
            }
            wsum[lane] = wi - ws;
        }
        __syncthreads();
        int excl = carry + wsum[warp] + inc - v;
        if (i < nb) counts[i] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void write_idx_kernel(const uint8_t* __restrict__ mask, int64_t n, const int* __restrict__ offsets,
                                 int32_t* idx) {
    __shared__ int warp_base[32];
    int64_t i = int64_t(blockIdx.x) * kCompactBlock + threadIdx.x;
    int v = i < n ? (mask[i] != 0) : 0;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned b = __ballot_sync(0xffffffffu, v);
    if (lane == 0) warp_base[warp] = __popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int w = 0; w < kCompactBlock / 32; ++w) {
            int c = warp_base[w];
            warp_base[w] = run;
            run += c;
        }
    }
    __syncthreads();
    if (v) {
        int pos = offsets[blockIdx.x] + warp_base[warp] + __popc(b & ((1u << lane) - 1u));
        idx[pos] = int32_t(i);
    }
}

// The row gathers and scatters below index with compacted sample indices; an
// index outside [0, rows) (a caller's bad count or index list) is skipped and
// raises the device flag's range bit instead of touching memory.
__global__ void gather_rows_kernel(float* dst, const float* __restrict__ src, int64_t src_rows,
                                   const int32_t* __restrict__ idx, const int32_t* count, int64_t n, int cols,
                                   int div, int* flag) {
    int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t cnt = *count < n ? *count : n;
    if (t >= cnt * cols) return;
    int64_t i = t / cols;
    int c = int(t % cols);
    int64_t row = idx[i];
    if (div > 1) row /= div;
    if (row < 0 || row >= src_rows) {
        raise_flag(flag, kFlagRange);
        return;
    }
    dst[t] = src[row * cols + c];
}

__global__ void scatter_rows_kernel(float* dst, int64_t dst_rows, const float* __restrict__ src,
                                    const int32_t* __restrict__ idx, const int32_t* count, int64_t n, int cols,
                                    int* flag) {
    int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t cnt = *count < n ? *count : n;
    if (t >= cnt * cols) return;
    int64_t i = t / cols;
    int c = int(t % cols);
    const int64_t row = idx[i];
    if (row < 0 || row >= dst_rows) {
        raise_flag(flag, kFlagRange);
        return;
    }
    dst[row * cols + c] = src[t];
}

__device__ __forceinline__ float softplus_f(float x) {
    // torch softplus (beta 1, threshold 20)
    return x > 20.f ? x : log1pf(expf(x));
}

__global__ void density_act_kernel(float* sigma, int64_t rows, const float* __restrict__ f,
                                   const int32_t* __restrict__ idx, const int32_t* count, int64_t n, int mode,
                                   float offset, int* flag) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t cnt = *count < n ? *count : n;
    if (i >= cnt) return;
    const int64_t row = idx[i];
    if (row < 0 || row >= rows) {
        raise_flag(flag, kFlagRange);
        return;
    }
    float x = f[i];
    sigma[row] = mode == 0 ? relu_f(x) : softplus_f(x + offset);
}

__global__ void density_act_bwd_kernel(float* df, const float* __restrict__ ds, int64_t rows,
                                       const float* __restrict__ f, const int32_t* __restrict__ idx,
                                       const int32_t* count, int64_t n, int mode, float offset, int* flag) {
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t cnt = *count < n ? *count : n;
    if (i >= cnt) return;
    const int64_t row = idx[i];
    if (row < 0 || row >= rows) {
        raise_flag(flag, kFlagRange);
        df[i] = 0.f;
        return;
    }
    float x = f[i];
    float g = ds[row];
    if (mode == 0) df[i] = x > 0.f ? g : 0.f;
    else {
        float y = x + offset;
        df[i] = y > 20.f ? g : g * sigmoid_f(y);
    }
}

// torch.linspace(0, 1, n)[i], the CPU formula the reference evaluates
// (SimpleTensoRF09.py:851-854): the first half counts up from 0, the second
// half down from 1.
__device__ __forceinline__ float linspace01(int i, int n) {
    if (n == 1) return 0.f;
    const float step = 1.f / float(n - 1);
    return i < n / 2 ? __fmul_rn(step, float(i)) : __fsub_rn(1.f, __fmul_rn(step, float(n - 1 - i)));
}

// LowRankTensor.update_alpha_mask's dense pass (SimpleTensoRF09.py:849-858 with
// compute_alpha :878-897): node (x, y, z) of the res[0] x res[1] x res[2] grid at
// xyz = lo (1 - s) + hi s, alpha = clamp(1 - exp(-sigma step), 0, 1), sigma the
// activated VM density, zero where the current alpha mask is empty.  Written
// z-major (alpha[z][y][x]), the transposed layout the mask volume keeps.
__global__ void alpha_grid_kernel(srf_vm_grid g, Box box, const float* __restrict__ vol, int vd, int vh, int vw,
                                  Box abox, float step, int mode, float offset, float* __restrict__ alpha) {
    const int gx = g.res[0], gy = g.res[1], gz = g.res[2];
    int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= int64_t(gx) * gy * gz) return;
    const int ix[3] = {int(t % gx), int((t / gx) % gy), int(t / (int64_t(gx) * gy))};
    float q[3], pn[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float s = linspace01(ix[a], g.res[a]);
        q[a] = __fadd_rn(__fmul_rn(box.lo[a], __fsub_rn(1.f, s)), __fmul_rn(box.hi[a], s));
    }
    bool keep = true;
    if (vol) {
        float an[3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
            an[a] = __fsub_rn(__fmul_rn((q[a] - abox.lo[a]) / (abox.hi[a] - abox.lo[a]), 2.f), 1.f);
        keep = alpha_positive(vol, vd, vh, vw, an[0], an[1], an[2]);
    }
    float sigma = 0.f;
    if (keep) {
#pragma unroll
        for (int a = 0; a < 3; ++a)
            pn[a] = __fsub_rn(__fmul_rn((q[a] - box.lo[a]) / (box.hi[a] - box.lo[a]), 2.f), 1.f);
        float acc = 0.f;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            Taps pt, lt;
            plane_taps(g, i, pn, pt, lt);
            acc = acc + vm_dot(g.planes[i], g.lines[i], g.n_comp[i], pt, lt);
        }
        sigma = mode == 0 ? relu_f(acc) : softplus_f(acc + offset);
    }
    float a = 1.f - expf(-sigma * step);
    alpha[t] = fminf(fmaxf(a, 0.f), 1.f);
}

// ---------------------------------------------------------------------------
// Deterministic scatter-add adjoint: every contribution w_c d line (or plane)
// value is rounded once to a 64-bit fixed-point integer with a power-of-two
// scale S and added with integer atomics, whose sums do not depend on the order
// of the additions; a last pass adds acc / S into the FP32 gradients.  With B the
// largest |d| times the largest |grid value| (bilinear weights are at most 1 and
// sum to 1) and at most n contributions per node (a point adds to each of its
// corners once), S = 2^floor(log2(2^62 / (n B))) keeps every partial sum inside
// 63 bits; each contribution is exact to 1 / (2 S) = n B 2^-63.
// Workspace: one int64 per grid element (planes then lines), then the scale
// (a double) and the two maxima (floats, as ordered integers).
// ---------------------------------------------------------------------------
struct FixedLayout {
    int64_t off[7];    // accumulator offsets of planes 0..2, lines 0..2, and the total
    size_t bytes;      // accumulators + scale + maxima
};

__host__ __device__ inline float* fixed_array(const srf_vm_grid& g, int k) {
    return k < 3 ? g.planes[k] : g.lines[k - 3];
}

FixedLayout fixed_layout(const srf_vm_grid& g) {
    FixedLayout L{};
    int64_t o = 0;
    for (int k = 0; k < 6; ++k) {
        L.off[k] = o;
        const int i = k % 3;
        o += k < 3 ? int64_t(g.res[kMatrixAxesHost[i][1]]) * g.res[kMatrixAxesHost[i][0]] * g.n_comp[i]
                   : int64_t(g.res[kVectorAxesHost[i]]) * g.n_comp[i];
    }
    L.off[6] = o;
    L.bytes = size_t(o) * 8 + 16;
    return L;
}

// maxima[0] = max |a| over na values, maxima[1] = max |grid value| (as float bits;
// non-negative floats order like their bit patterns)
__global__ void fixed_absmax_kernel(const float* __restrict__ a, int64_t na, srf_vm_grid g, FixedLayout L,
                                    unsigned int* maxima) {
    float ma = 0.f, mg = 0.f;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < na; i += stride) ma = fmaxf(ma, fabsf(a[i]));
    for (int k = 0; k < 6; ++k) {
        const float* src = fixed_array(g, k);
        const int64_t cnt = L.off[k + 1] - L.off[k];
        for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < cnt; i += stride)
            mg = fmaxf(mg, fabsf(src[i]));
    }
    for (int o = 16; o > 0; o >>= 1) {
        ma = fmaxf(ma, __shfl_xor_sync(0xffffffffu, ma, o));
        mg = fmaxf(mg, __shfl_xor_sync(0xffffffffu, mg, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(maxima, __float_as_uint(ma));
        atomicMax(maxima + 1, __float_as_uint(mg));
    }
}

__global__ void fixed_scale_kernel(const unsigned int* maxima, int64_t n, double* scale) {
    const double b = double(__uint_as_float(maxima[0])) * double(__uint_as_float(maxima[1]));
    const double bound = b * double(n > 0 ? n : 1);
    // the largest power of two S with S * bound <= 2^62 (1 for an all-zero bound)
    int e = 0;
    if (bound > 0.0 && isfinite(bound)) {
        frexp(bound, &e);            // bound < 2^e
        e = 62 - e;
    }
    *scale = ldexp(1.0, e);
}

__device__ __forceinline__ void fixed_add(int64_t* acc, float v, double scale) {
    if (v != 0.f)
        atomicAdd(reinterpret_cast<unsigned long long*>(acc), (unsigned long long)llrint(double(v) * scale));
}

__global__ void vm_bwd_fixed_kernel(srf_vm_grid g, const float* __restrict__ pts, int64_t n,
                                    const float* __restrict__ dfeat, int ld, int per_component, FixedLayout L,
                                    int64_t* acc, const double* scale_dev) {
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const double scale = *scale_dev;
    const float* q = pts + 3 * p;
    const float ds = per_component ? 0.f : dfeat[p];
    if (!per_component && ds == 0.f) return;
    int off = 0;
    for (int i = 0; i < 3; ++i) {
        Taps pt, lt;
        plane_taps(g, i, q, pt, lt);
        const int R = g.n_comp[i];
        const float* pl = g.planes[i];
        const float* ln = g.lines[i];
        int64_t* apl = acc + L.off[i];
        int64_t* aln = acc + L.off[3 + i];
        for (int r = 0; r < R; ++r) {
            float pv = 0.f, lv = 0.f;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (pt.idx[c] >= 0) pv += pl[int64_t(pt.idx[c]) * R + r] * pt.w[c];
                if (lt.idx[c] >= 0) lv += ln[int64_t(lt.idx[c]) * R + r] * lt.w[c];
            }
            const float d = per_component ? dfeat[p * ld + off + r] : ds;
            const float dp = d * lv, dl = d * pv;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                if (pt.idx[c] >= 0) fixed_add(apl + int64_t(pt.idx[c]) * R + r, dp * pt.w[c], scale);
                if (lt.idx[c] >= 0) fixed_add(aln + int64_t(lt.idx[c]) * R + r, dl * lt.w[c], scale);
            }
        }
        off += R;
    }
}

// grad += acc / S over every grid element
__global__ void fixed_to_grad_kernel(srf_vm_grid gg, FixedLayout L, const int64_t* __restrict__ acc,
                                     const double* scale_dev) {
    const double inv = 1.0 / *scale_dev;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < L.off[6]; e += stride) {
        int k = 0;
        while (k < 5 && e >= L.off[k + 1]) ++k;
        fixed_array(gg, k)[e - L.off[k]] += float(double(acc[e]) * inv);
    }
}

int vm_bwd_fixed(const srf_vm_grid& gg, const srf_vm_grid& g, const float* pts, int64_t n, const float* dfeat,
                 int ld, int per_component, void* ws, size_t ws_bytes, cudaStream_t s) {
    const FixedLayout L = fixed_layout(g);
    if (!ws || ws_bytes < L.bytes) return SRF_ERR_WORKSPACE;
    if ((reinterpret_cast<uintptr_t>(ws) & 15u) != 0) return SRF_ERR_ALIGN;
    int64_t* acc = static_cast<int64_t*>(ws);
    double* scale = reinterpret_cast<double*>(acc + L.off[6]);
    unsigned int* maxima = reinterpret_cast<unsigned int*>(scale + 1);
    cudaError_t e = cudaMemsetAsync(ws, 0, L.bytes, s);
    if (e != cudaSuccess) {
        set_cuda_error(e);
        return SRF_ERR_CUDA;
    }
    fixed_absmax_kernel<<<grid_1d(1 << 20, 256), 256, 0, s>>>(dfeat, n * (per_component ? ld : 1), g, L, maxima);
    if (int st = launch_status()) return st;
    fixed_scale_kernel<<<1, 1, 0, s>>>(maxima, n, scale);
    if (int st = launch_status()) return st;
    vm_bwd_fixed_kernel<<<grid_1d(n, 128), 128, 0, s>>>(g, pts, n, dfeat, ld, per_component, L, acc, scale);
    if (int st = launch_status()) return st;
    const int64_t conv = L.off[6] < (int64_t(1) << 22) ? L.off[6] : (int64_t(1) << 22);
    if (conv > 0) fixed_to_grad_kernel<<<grid_1d(conv, 256), 256, 0, s>>>(gg, L, acc, scale);
    return launch_status();
}

int check_grid(const srf_vm_grid* g, bool need) {
    if (!g) return SRF_ERR_NULL;
    for (int i = 0; i < 3; ++i) {
        if (need && (!g->planes[i] || !g->lines[i])) return SRF_ERR_NULL;
        if (g->res[i] < 1 || g->n_comp[i] < 0 || g->n_comp[i] > 1024) return SRF_ERR_SHAPE;
        if ((g->n_comp[i] & 3) == 0 && (!aligned16(g->planes[i]) || !aligned16(g->lines[i]))) return SRF_ERR_ALIGN;
    }
    return SRF_OK;
}

}  // namespace
}  // namespace srf

using namespace srf;

extern "C" int srf_vm_density_forward(const srf_vm_grid* grid, const float* pts, int64_t n_pts, float* features,
                                      void* stream) {
    int st = check_grid(grid, true);
    if (st) return st;
    if (!pts || !features) return SRF_ERR_NULL;
    if (n_pts < 0) return SRF_ERR_SHAPE;
    if (n_pts == 0) return SRF_OK;
    density_fwd_kernel<<<grid_1d(n_pts, 128), 128, 0, as_stream(stream)>>>(*grid, pts, n_pts, features);
    return launch_status();
}

extern "C" int srf_vm_density_backward(const srf_vm_grid* grad_grid, const srf_vm_grid* grid, const float* pts,
                                       int64_t n_pts, const float* d_features, void* stream) {
    int st = check_grid(grid, true);
    if (st) return st;
    if ((st = check_grid(grad_grid, true))) return st;
    if (!pts || !d_features) return SRF_ERR_NULL;
    if (n_pts <= 0) return n_pts < 0 ? SRF_ERR_SHAPE : SRF_OK;
    for (int i = 0; i < 3; ++i)
        if (grad_grid->n_comp[i] != grid->n_comp[i] || grad_grid->res[i] != grid->res[i]) return SRF_ERR_SHAPE;
    const int G = group_lanes(*grid);
    if (G) {
        return launch_grouped(G, n_pts, [&](auto gc) {
            constexpr int g = decltype(gc)::value;
            vm_bwd_group_kernel<g><<<grid_1d(n_pts * g, 128), 128, 0, as_stream(stream)>>>(*grad_grid, *grid, pts,
                                                                                           n_pts, d_features, 1, 0);
            return launch_status();
        });
    }
    vm_bwd_kernel<<<grid_1d(n_pts, 128), 128, 0, as_stream(stream)>>>(*grad_grid, *grid, pts, n_pts, d_features, 1, 0);
    return launch_status();
}

extern "C" int srf_vm_color_forward(const srf_vm_grid* grid, const float* pts, int64_t n_pts, float* features,
                                    void* stream) {
    int st = check_grid(grid, true);
    if (st) return st;
    if (!pts || !features) return SRF_ERR_NULL;
    if (n_pts <= 0) return n_pts < 0 ? SRF_ERR_SHAPE : SRF_OK;
    int ld = grid->n_comp[0] + grid->n_comp[1] + grid->n_comp[2];
    const int G = group_lanes(*grid);
    // candidates: every group size that divides the component counts (G, G/2, ..., 1),
    // then the per-thread kernel; the tuner times them per (R0, R1, R2)
    int cand[6], nc = 0;
    if (G && (ld & 3) == 0 && aligned16(features))
        for (int g = G; g >= 1; g >>= 1) cand[nc++] = g;
    cand[nc++] = 0;
    auto run = [&](int i) -> int {
        const int g = cand[i];
        if (g == 0) {
            color_fwd_kernel<<<grid_1d(n_pts, 128), 128, 0, as_stream(stream)>>>(*grid, pts, n_pts, ld, features);
            return launch_status();
        }
        return launch_grouped(g, n_pts, [&](auto gc) {
            constexpr int gg = decltype(gc)::value;
            color_fwd_group_kernel<gg><<<grid_1d(n_pts * gg, 128), 128, 0, as_stream(stream)>>>(*grid, pts, n_pts,
                                                                                                ld, features);
            return launch_status();
        });
    };
    const tune::Key key{tune::kSiteVmColorGroup, grid->n_comp[0], grid->n_comp[1], grid->n_comp[2]};
    return run(tune::pick(key, nc, 0, as_stream(stream), run));
}

extern "C" int srf_vm_color_backward(const srf_vm_grid* grad_grid, const srf_vm_grid* grid, const float* pts,
                                     int64_t n_pts, const float* d_features, void* stream) {
    int st = check_grid(grid, true);
    if (st) return st;
    if ((st = check_grid(grad_grid, true))) return st;
    if (!pts || !d_features) return SRF_ERR_NULL;
    if (n_pts <= 0) return n_pts < 0 ? SRF_ERR_SHAPE : SRF_OK;
    for (int i = 0; i < 3; ++i)
        if (grad_grid->n_comp[i] != grid->n_comp[i] || grad_grid->res[i] != grid->res[i]) return SRF_ERR_SHAPE;
    int ld = grid->n_comp[0] + grid->n_comp[1] + grid->n_comp[2];
    // rows of d_features are read 16 bytes at a time when ld is a multiple of 4
    if ((ld & 3) == 0 && !aligned16(d_features)) return SRF_ERR_ALIGN;
    const int G = group_lanes(*grid);
    if (G) {   // G != 0 implies ld % 4 == 0; d_features alignment is checked above
        return launch_grouped(G, n_pts, [&](auto gc) {
            constexpr int g = decltype(gc)::value;
            vm_bwd_group_kernel<g><<<grid_1d(n_pts * g, 128), 128, 0, as_stream(stream)>>>(*grad_grid, *grid, pts,
                                                                                           n_pts, d_features, ld, 1);
            return launch_status();
        });
    }
    vm_bwd_kernel<<<grid_1d(n_pts, 128), 128, 0, as_stream(stream)>>>(*grad_grid, *grid, pts, n_pts, d_features, ld, 1);
    return launch_status();
}

extern "C" size_t srf_vm_backward_fixed_workspace_size(const srf_vm_grid* grid) {
    if (check_grid(grid, false)) return 0;
    return fixed_layout(*grid).bytes;
}

// The deterministic adjoints (fixed-point integer accumulation): same arguments as
// srf_vm_density_backward / srf_vm_color_backward plus the workspace.
extern "C" int srf_vm_density_backward_fixed(const srf_vm_grid* grad_grid, const srf_vm_grid* grid, const float* pts,
                                             int64_t n_pts, const float* d_features, void* workspace,
                                             size_t workspace_bytes, void* stream) {
    int st = check_grid(grid, true);
    if (st) return st;
    if ((st = check_grid(grad_grid, true))) return st;
    if (!pts || !d_features) return SRF_ERR_NULL;
    if (n_pts <= 0) return n_pts < 0 ? SRF_ERR_SHAPE : SRF_OK;
    for (int i = 0; i < 3; ++i)
        if (grad_grid->n_comp[i] != grid->n_comp[i] || grad_grid->res[i] != grid->res[i]) return SRF_ERR_SHAPE;
    return vm_bwd_fixed(*grad_grid, *grid, pts, n_pts, d_features, 1, 0, workspace, workspace_bytes, as_stream(stream));
}

extern "C" int srf_vm_color_backward_fixed(const srf_vm_grid* grad_grid, const srf_vm_grid* grid, const float* pts,
                                           int64_t n_pts, const float* d_features, void* workspace,
                                           size_t workspace_bytes, void* stream) {
    int st = check_grid(grid, true);
    if (st) return st;
    if ((st = check_grid(grad_grid, true))) return st;
    if (!pts || !d_features) return SRF_ERR_NULL;
    if (n_pts <= 0) return n_pts < 0 ? SRF_ERR_SHAPE : SRF_OK;
    for (int i = 0; i < 3; ++i)
        if (grad_grid->n_comp[i] != grid->n_comp[i] || grad_grid->res[i] != grid->res[i]) return SRF_ERR_SHAPE;
    const int ld = grid->n_comp[0] + grid->n_comp[1] + grid->n_comp[2];
    return vm_bwd_fixed(*grad_grid, *grid, pts, n_pts, d_features, ld, 1, workspace, workspace_bytes,
                        as_stream(stream));
}

extern "C" int srf_tensorf_sample_mask(const float* rays_o, const float* rays_d, const float* z, int n_rays,
                                       int n_samples, const float* bbox, const float* alpha_volume, int vol_d,
                                       int vol_h, int vol_w, const float* alpha_bbox, float* pts_norm, uint8_t* mask,
                                       void* stream) {
    if (!rays_o || !rays_d || !z || !bbox || !pts_norm || !mask) return SRF_ERR_NULL;
    if (alpha_volume && !alpha_bbox) return SRF_ERR_NULL;
    if (n_rays < 0 || n_samples < 1) return SRF_ERR_SHAPE;
    if (alpha_volume && (vol_d < 1 || vol_h < 1 || vol_w < 1)) return SRF_ERR_SHAPE;
    if (n_rays == 0) return SRF_OK;
    Box b{{bbox[0], bbox[1], bbox[2]}, {bbox[3], bbox[4], bbox[5]}};
    Box ab = b;
    if (alpha_bbox) ab = Box{{alpha_bbox[0], alpha_bbox[1], alpha_bbox[2]}, {alpha_bbox[3], alpha_bbox[4], alpha_bbox[5]}};
    int64_t tot = int64_t(n_rays) * n_samples;
    sample_mask_kernel<<<grid_1d(tot, 256), 256, 0, as_stream(stream)>>>(rays_o, rays_d, z, n_rays, n_samples, b,
                                                                        alpha_volume, vol_d, vol_h, vol_w, ab,
                                                                        pts_norm, mask);
    return launch_status();
}

extern "C" int srf_alpha_mask_query(const float* alpha_volume, int vol_d, int vol_h, int vol_w, const float* pts_norm,
                                    int64_t n_pts, uint8_t* out, void* stream) {
    if (!alpha_volume || !pts_norm || !out) return SRF_ERR_NULL;
    if (vol_d < 1 || vol_h < 1 || vol_w < 1 || n_pts < 0) return SRF_ERR_SHAPE;
    if (n_pts == 0) return SRF_OK;
    alpha_query_kernel<<<grid_1d(n_pts, 256), 256, 0, as_stream(stream)>>>(alpha_volume, vol_d, vol_h, vol_w,
                                                                          pts_norm, n_pts, out);
    return launch_status();
}

extern "C" size_t srf_compact_workspace_size(int64_t n) {
    if (n < 0) return 0;
    return size_t((n + kCompactBlock - 1) / kCompactBlock + 1) * sizeof(int);
}

extern "C" int srf_compact(const uint8_t* mask, int64_t n, int32_t* idx, int32_t* count_dev, void* workspace,
                           size_t workspace_bytes, void* stream) {
    if (!mask || !idx || !count_dev) return SRF_ERR_NULL;
    if (n < 0 || n > 0x7fffffff) return SRF_ERR_SHAPE;
    cudaStream_t s = as_stream(stream);
    if (n == 0) {
        cudaError_t e = cudaMemsetAsync(count_dev, 0, sizeof(int32_t), s);
        return e == cudaSuccess ? SRF_OK : SRF_ERR_CUDA;
    }
    if (!workspace || workspace_bytes < srf_compact_workspace_size(n)) return SRF_ERR_WORKSPACE;
    int nb = int((n + kCompactBlock - 1) / kCompactBlock);
    int* counts = static_cast<int*>(workspace);
    count_kernel<<<nb, kCompactBlock, 0, s>>>(mask, n, counts);
    int st = launch_status();
    if (st) return st;
    scan_counts_kernel<<<1, 1024, 0, s>>>(counts, nb, count_dev);
    if ((st = launch_status())) return st;
    write_idx_kernel<<<nb, kCompactBlock, 0, s>>>(mask, n, counts, idx);
    return launch_status();
}

// ---------------------------------------------------------------------------
// Compaction without any caller-provided or library-allocated memory.
//
// srf_compact needs a small scratch buffer (one int per 1024 mask elements) that
// the caller allocates.  Some callers cannot allocate device memory at all: a
// plugin that runs inside another framework's fixed memory pool, code holding a
// no-allocation guarantee (a real-time loop where cudaMalloc's implicit device
// synchronisation is not acceptable), or a thin foreign-language binding that
// only has the mask and output pointers.  For them the scratch below is a fixed
// array compiled into this library: every GPU that loads the library keeps
// these 64 KB until the process exits.
// ---------------------------------------------------------------------------
static __device__ __align__(256) int g_compact_noalloc_scratch[SRF_COMPACT_NOALLOC_MAX_BLOCKS];

namespace {

// The array's name is only a host-side handle in host code; the device address
// comes from cudaGetSymbolAddress, looked up once per device with that device
// current and cached.
int* compact_noalloc_scratch(int* status) {
    static std::mutex mu;
    static int* cache[64] = {nullptr};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) {
        if (e != cudaSuccess) set_cuda_error(e);
        *status = SRF_ERR_CUDA;
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (!cache[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_compact_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_cuda_error(e);
            *status = SRF_ERR_CUDA;
            return nullptr;
        }
        cache[dev] = static_cast<int*>(p);
    }
    *status = SRF_OK;
    return cache[dev];
}

}  // namespace

extern "C" int srf_compact_noalloc(const uint8_t* mask, int64_t n, int32_t* idx, int32_t* count_dev, void* stream) {
    if (!mask || !idx || !count_dev) return SRF_ERR_NULL;
    if (n < 0 || n > int64_t(SRF_COMPACT_NOALLOC_MAX_ELEMENTS)) return SRF_ERR_SHAPE;
    cudaStream_t s = as_stream(stream);
    if (n == 0) {
        cudaError_t e = cudaMemsetAsync(count_dev, 0, sizeof(int32_t), s);
        if (e != cudaSuccess) set_cuda_error(e);
        return e == cudaSuccess ? SRF_OK : SRF_ERR_CUDA;
    }
    int st = SRF_OK;
    int* scratch = compact_noalloc_scratch(&st);
    if (!scratch) return st;
    // Each call writes every scratch entry it later reads (one count per block,
    // then the in-place scan), so leftovers of an earlier call never leak in.
    int nb = int((n + kCompactBlock - 1) / kCompactBlock);
    count_kernel<<<nb, kCompactBlock, 0, s>>>(mask, n, scratch);
    if ((st = launch_status())) return st;
    scan_counts_kernel<<<1, 1024, 0, s>>>(scratch, nb, count_dev);
    if ((st = launch_status())) return st;
    write_idx_kernel<<<nb, kCompactBlock, 0, s>>>(mask, n, scratch, idx);
    return launch_status();
}

extern "C" int srf_threshold_mask(const float* x, int64_t n, float threshold, uint8_t* mask, void* stream) {
    if (!x || !mask) return SRF_ERR_NULL;
    if (n < 0) return SRF_ERR_SHAPE;
    if (n == 0) return SRF_OK;
    threshold_kernel<<<grid_1d(n, 256), 256, 0, as_stream(stream)>>>(x, n, threshold, mask);
    return launch_status();
}

extern "C" int srf_gather_rows(float* dst, const float* src, int64_t src_rows, const int32_t* idx,
                               const int32_t* count_dev, int64_t n, int cols, int src_row_div, void* stream) {
    if (!dst || !src || !idx || !count_dev) return SRF_ERR_NULL;
    if (n < 0 || cols < 1 || src_row_div < 1 || src_rows < 0) return SRF_ERR_SHAPE;
    if (n == 0) return SRF_OK;
    gather_rows_kernel<<<grid_1d(n * cols, 256), 256, 0, as_stream(stream)>>>(dst, src, src_rows, idx, count_dev, n,
                                                                              cols, src_row_div, device_flag());
    return launch_status();
}

extern "C" int srf_scatter_rows(float* dst, int64_t dst_rows, const float* src, const int32_t* idx,
                                const int32_t* count_dev, int64_t n, int cols, void* stream) {
    if (!dst || !src || !idx || !count_dev) return SRF_ERR_NULL;
    if (n < 0 || cols < 1 || dst_rows < 0) return SRF_ERR_SHAPE;
    if (n == 0) return SRF_OK;
    scatter_rows_kernel<<<grid_1d(n * cols, 256), 256, 0, as_stream(stream)>>>(dst, dst_rows, src, idx, count_dev, n,
                                                                               cols, device_flag());
    return launch_status();
}

extern "C" int srf_density_activation(float* sigma_dense, int64_t rows, const float* features, const int32_t* idx,
                                      const int32_t* count_dev, int64_t n, int mode, float offset, void* stream) {
    if (!sigma_dense || !features || !idx || !count_dev) return SRF_ERR_NULL;
    if (n < 0 || mode < 0 || mode > 1 || rows < 0) return SRF_ERR_SHAPE;
    if (n == 0) return SRF_OK;
    density_act_kernel<<<grid_1d(n, 256), 256, 0, as_stream(stream)>>>(sigma_dense, rows, features, idx, count_dev, n,
                                                                      mode, offset, device_flag());
    return launch_status();
}

extern "C" int srf_density_activation_backward(float* d_features, const float* d_sigma_dense, int64_t rows,
                                               const float* features, const int32_t* idx, const int32_t* count_dev,
                                               int64_t n, int mode, float offset, void* stream) {
    if (!d_features || !d_sigma_dense || !features || !idx || !count_dev) return SRF_ERR_NULL;
    if (n < 0 || mode < 0 || mode > 1 || rows < 0) return SRF_ERR_SHAPE;
    if (n == 0) return SRF_OK;
    density_act_bwd_kernel<<<grid_1d(n, 256), 256, 0, as_stream(stream)>>>(d_features, d_sigma_dense, rows, features,
                                                                          idx, count_dev, n, mode, offset,
                                                                          device_flag());
    return launch_status();
}

// ---------------------------------------------------------------- CP lines --

static int check_cp_grid(const srf_vm_grid* g) {
    if (!g) return SRF_ERR_NULL;
    for (int i = 0; i < 3; ++i) {
        if (!g->lines[i]) return SRF_ERR_NULL;
        if (g->res[i] < 1 || g->n_comp[i] != g->n_comp[0] || g->n_comp[0] < 1 || g->n_comp[0] > 1024)
            return SRF_ERR_SHAPE;
    }
    return SRF_OK;
}

static int cp_forward(const srf_vm_grid* grid, const float* pts, int64_t n_pts, float* features, int per_component,
                      void* stream) {
    int st = check_cp_grid(grid);
    if (st) return st;
    if (n_pts < 0) return SRF_ERR_SHAPE;
    if (n_pts == 0) return SRF_OK;
    if (!pts || !features) return SRF_ERR_NULL;
    cp_fwd_kernel<<<grid_1d(n_pts, 128), 128, 0, as_stream(stream)>>>(*grid, pts, n_pts, per_component, features);
    return launch_status();
}

static int cp_backward(const srf_vm_grid* grad_grid, const srf_vm_grid* grid, const float* pts, int64_t n_pts,
                       const float* d_features, int per_component, void* stream) {
    int st = check_cp_grid(grid);
    if (st) return st;
    if ((st = check_cp_grid(grad_grid))) return st;
    for (int i = 0; i < 3; ++i)
        if (grad_grid->n_comp[i] != grid->n_comp[i] || grad_grid->res[i] != grid->res[i]) return SRF_ERR_SHAPE;
    if (n_pts < 0) return SRF_ERR_SHAPE;
    if (n_pts == 0) return SRF_OK;
    if (!pts || !d_features) return SRF_ERR_NULL;
    cp_bwd_kernel<<<grid_1d(n_pts, 128), 128, 0, as_stream(stream)>>>(*grad_grid, *grid, pts, n_pts, d_features,
                                                                   per_component);
    return launch_status();
}

extern "C" int srf_cp_density_forward(const srf_vm_grid* grid, const float* pts, int64_t n_pts, float* features,
                                      void* stream) {
    return cp_forward(grid, pts, n_pts, features, 0, stream);
}

extern "C" int srf_cp_density_backward(const srf_vm_grid* grad_grid, const srf_vm_grid* grid, const float* pts,
                                       int64_t n_pts, const float* d_features, void* stream) {
    return cp_backward(grad_grid, grid, pts, n_pts, d_features, 0, stream);
}

extern "C" int srf_cp_color_forward(const srf_vm_grid* grid, const float* pts, int64_t n_pts, float* features,
                                    void* stream) {
    return cp_forward(grid, pts, n_pts, features, 1, stream);
}

extern "C" int srf_cp_color_backward(const srf_vm_grid* grad_grid, const srf_vm_grid* grid, const float* pts,
                                     int64_t n_pts, const float* d_features, void* stream) {
    return cp_backward(grad_grid, grid, pts, n_pts, d_features, 1, stream);
}

extern "C" int srf_vm_alpha_grid(const srf_vm_grid* grid, const float* bbox, const float* alpha_volume, int vol_d,
                                 int vol_h, int vol_w, const float* alpha_bbox, float step, int density_mode,
                                 float density_offset, float* alpha, void* stream) {
    int st = check_grid(grid, true);
    if (st) return st;
    if (!bbox || !alpha || (alpha_volume && !alpha_bbox)) return SRF_ERR_NULL;
    if (alpha_volume && (vol_d < 1 || vol_h < 1 || vol_w < 1)) return SRF_ERR_SHAPE;
    if (density_mode != 0 && density_mode != 1) return SRF_ERR_SHAPE;
    Box b{{bbox[0], bbox[1], bbox[2]}, {bbox[3], bbox[4], bbox[5]}};
    Box ab{};
    if (alpha_bbox) ab = Box{{alpha_bbox[0], alpha_bbox[1], alpha_bbox[2]}, {alpha_bbox[3], alpha_bbox[4], alpha_bbox[5]}};
    int64_t n = int64_t(grid->res[0]) * grid->res[1] * grid->res[2];
    alpha_grid_kernel<<<grid_1d(n, 256), 256, 0, as_stream(stream)>>>(*grid, b, alpha_volume, vol_d, vol_h, vol_w, ab,
                                                                     step, density_mode, density_offset, alpha);
    return launch_status();
}
