// Internal: layout of one NeRF MLP (SimpleNeRF17.py:616-667) shared by the FP32
// and BF16 implementations.
#pragma once

#include <string>
#include <utility>
#include <vector>

#include "gemm_simt.cuh"

namespace srf {

struct MlpLayout {
    srf_nerf_mlp_desc desc;
    int Dp, Wp, Dv, Wv;
    int ppe;    // width of the xyz encoding, 3(2L+1)
    int pin;    // trunk input width (== ppe unless the points-augmentation variant)
    int vpe;    // width of the view-direction encoding (0 without view dirs)
    int vin;    // extra inputs of the first view layer besides the feature
    bool vdep;  // view-dependent rgb head
    int skip;
    bool valid;
    std::vector<int> layer_k, view_k;                 // input widths of trunk / view layers
    std::vector<std::string> names;                   // reference state_dict names, in order
    std::vector<std::pair<int, int>> shapes;          // (rows, cols); cols 0 for a bias

    explicit MlpLayout(const srf_nerf_mlp_desc& d);
    int idx_trunk_w(int j) const;
    int idx_view_w(int j) const;
    int idx_out_w() const;
    int idx_feat_w() const;
    int idx_rgb_w() const;
    SegRows trunk_input(int j, const float* enc, float* const* h) const;
    SegRows view_input(int j, const float* feat, const float* enc, const float* encv, int dir_div,
                       float* const* hv) const;
};

size_t mlp_tc_workspace(const MlpLayout& L, int64_t m, bool bwd);
// fmt: tc::kFmtBF16 (0) or tc::kFmtF16 (1); scaler: optional in the forward, required by the FP16 backward
int mlp_tc_forward(const MlpLayout& L, const float* const* P, const float* pts, const float* dirs, int dir_div,
                   int64_t m, const float* noise, float* sigma, float* rgb, bool bwd, void* ws, size_t ws_bytes,
                   int fmt, srf_loss_scaler* scaler, cudaStream_t s);
int mlp_tc_backward(const MlpLayout& L, const float* const* P, const float* dsigma, const float* drgb, int64_t m,
                    int dir_div, float* const* G, void* ws, size_t ws_bytes, int fmt, srf_loss_scaler* scaler,
                    cudaStream_t s);

}  // namespace srf
