/*
 * srf_gb300.h -- C ABI of the GB300-native Simple-RF rendering hot path.
 *
 * Every entry point takes caller-owned device pointers, explicit sizes, an
 * explicit CUDA stream (as `void*`, a cudaStream_t) and, where it needs
 * temporaries, a caller-provided workspace.  The library never allocates device
 * memory and never frees caller memory.  The compute entry points are stateless
 * and re-entrant; the process-wide state is the device error flag, the path
 * switches (srf_nerf_mlp_fused_path, srf_tensorf_basis_adjoint_path), the tile
 * tuner's table (srf_autotune_*) and srf_compact_noalloc's fixed scratch array.
 * Work is enqueued on the given stream only (so calls are legal inside CUDA
 * stream capture).  Return value: SRF_OK (0) or an srf_status code; no
 * exceptions cross this boundary and no device code traps.
 *
 * Reference citations are `file:line` inside the Simple-RF project
 * (NagabhushanSN95/Simple-RF, src/...).
 */
#ifndef SRF_GB300_H
#define SRF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SRF_OK = 0,
    SRF_ERR_NULL = 1,          /* a required pointer is NULL                      */
    SRF_ERR_SHAPE = 2,         /* a size / dimension is out of the supported range */
    SRF_ERR_ALIGN = 3,         /* a pointer or stride breaks an alignment rule     */
    SRF_ERR_WORKSPACE = 4,     /* workspace smaller than srf_*_workspace_size()    */
    SRF_ERR_CUDA = 5,          /* a CUDA launch or runtime call failed             */
    SRF_ERR_TIMEOUT = 6,       /* a bounded device-side wait gave up               */
    SRF_ERR_RANGE = 7,         /* a device-side index check failed (see flag)      */
    SRF_ERR_UNSUPPORTED = 8    /* configuration valid in the reference, not here   */
} srf_status;

/* Library utilities, no reference counterpart.  Human-readable name of a status
 * code (static string). */
const char* srf_status_string(int status);
/* Library version, e.g. "srf_gb300 1.0 sm_103a" (no reference counterpart). */
const char* srf_version(void);
/* Text of the last CUDA error seen by this thread (static thread-local buffer;
 * no reference counterpart). */
const char* srf_last_cuda_error(void);
/* Number of kernels this library has launched (or captured into a graph) in
 * this process; used to count launches per training step (no reference
 * counterpart). */
int64_t srf_launch_count(void);

/* Read-bandwidth probe (a measurement utility; no counterpart in the reference):
 * streams `bytes` (multiple of 16, 16-byte aligned) of `buf` `passes` times with
 * 16-byte loads and writes one float per block to sink (srf_read_probe_blocks()
 * floats).  A buffer that fits in L2 gives the L2 read rate that bounds the VM
 * plane gathers (their planes stay L2-resident); a larger one the HBM read rate. */
int srf_read_probe_blocks(void);
int srf_read_probe(const void* buf, int64_t bytes, int passes, float* sink, void* stream);
/* Reads and clears the device-side error flag (bounded-wait timeouts, index
 * range violations) that kernels set instead of trapping.  Synchronises `stream`.
 * Writes the flag value (0 = clean) to *flag_out. */
int srf_read_device_flag(int* flag_out, void* stream);
/* A non-blocking CUDA stream of the current device, and its release (the
 * release returns at once; pending work finishes first).  Concurrent stages of a
 * step (an augmented net's pass, the coarse net's backward) need streams that
 * are distinct CUDA streams; pooled streams of a host framework may alias one
 * another.  No reference counterpart (the reference
 * runs on PyTorch's current stream). */
int srf_stream_create(void** stream_out);
int srf_stream_destroy(void* stream);

/* ------------------------------------------------------------------------ */
/* Ray generation and sampling                                               */
/* ------------------------------------------------------------------------ */

/* World rays of pixels: pixel_id (N,3) int32 (image, x, y), intrinsics (N,3,3),
 * extrinsics (N,4,4) camera-to-world; half_pixel adds 0.5 to x and y (the
 * reference's mip_nerf_used flag).  Replaces CommonUtils04.get_rays_tr
 * (src/utils/CommonUtils04.py:73-95, non-synthetic branch). */
int srf_pixel_rays(const int32_t* pixel_id, const float* intrinsics, const float* extrinsics, int n_rays,
                   int half_pixel, float* rays_o, float* rays_d, void* stream);

/* NDC warp + view directions of world rays.
 * Replaces CommonUtils04.get_ndc_rays_tr (src/utils/CommonUtils04.py:120-138)
 * and get_view_dirs_tr (:147-149).  fx, fy per ray (N,); any output may be NULL. */
int srf_ndc_rays(const float* rays_o, const float* rays_d, const float* fx, const float* fy, int n_rays,
                 int height, int width, float near_plane, float* rays_o_ndc, float* rays_d_ndc,
                 float* view_dirs, void* stream);

/* Stratified coarse depths z (N,S).  u (N,S) uniforms or NULL (no jitter).
 * Replaces SimpleNeRF.get_z_vals_coarse (src/models/SimpleNeRF17.py:330-358). */
int srf_stratified_z(float* z, const float* u, int n_rays, int n_samples, float near_plane, float far_plane,
                     int lindisp, void* stream);

/* Inverse-CDF samples (N,n_samples) from bins (N,n_bins) and weights (N,n_bins-1);
 * u (N,n_samples) uniforms or NULL for the deterministic linspace(0,1).
 * Replaces SimpleNeRF.sample_pdf (src/models/SimpleNeRF17.py:384-417; identical
 * copy SimpleTensoRF09.py:427-460); searchsorted(right=True) bin semantics. */
int srf_sample_pdf(float* samples, const float* bins, const float* weights, const float* u, int n_rays,
                   int n_bins, int n_samples, void* stream);

/* Fine depths: mids of z_coarse, sample_pdf on weights_coarse[:,1:-1], merged and
 * sorted with z_coarse -> z_fine (N, n_coarse+n_fine).  n_coarse+n_fine <= 1024.
 * Replaces SimpleNeRF.get_z_vals_fine (src/models/SimpleNeRF17.py:360-371). */
int srf_fine_z(float* z_fine, const float* z_coarse, const float* weights_coarse, const float* u, int n_rays,
               int n_coarse, int n_fine, void* stream);

/* TensoRF AABB ray marching depths z (N,S) = t_min + step*(arange(S) + u_ray).
 * u (N,) or NULL.  Replaces SimpleTensoRF.get_z_vals_coarse non-NDC branch
 * (src/models/SimpleTensoRF09.py:388-400). */
int srf_aabb_z(float* z, const float* rays_o, const float* rays_d, const float* u, int n_rays, int n_samples,
               const float* bbox /* host (2,3) */, float near_plane, float far_plane, float step_size,
               void* stream);

/* Positional encoding [x, sin(2^0 x), cos(2^0 x), ...] of x (M,dims) into
 * out (M, ld_out) columns [0, dims*(2L+1)).
 * Replaces PositionalEncoder (src/models/SimpleNeRF17.py:581-613). */
int srf_positional_encoding(float* out, int ld_out, const float* x, int64_t m, int dims, int degree, void* stream);

/* ------------------------------------------------------------------------ */
/* NeRF MLP (fused PE + trunk + heads), forward and backward                 */
/* ------------------------------------------------------------------------ */

typedef struct {
    int points_net_depth;        /* Dp (reference: points_net_depth)             */
    int points_net_width;        /* Wp                                           */
    int views_net_depth;         /* Dv                                           */
    int views_net_width;         /* Wv                                           */
    int points_pe_degree;        /* L for xyz                                    */
    int views_pe_degree;         /* L for view directions                        */
    int points_sigma_pe_degree;  /* -1 when absent (points-augmentation variant) */
    int use_view_dirs;
    int view_dependent_rgb;
    int skip_layer;              /* 4: concat [input, h] after this layer        */
} srf_nerf_mlp_desc;

/* FP32: the plain path (SIMT, FP32 throughout).  BF16 / FP16: tcgen05 tensor
 * cores with FP32 master weights and FP32 accumulation, 16-bit operands of that
 * format.  FP16 keeps 3 more mantissa bits (forward activations are the dominant
 * source of gradient error) and its backward runs on loss-scaled gradients:
 * it needs an srf_loss_scaler. */
enum { SRF_PRECISION_FP32 = 0, SRF_PRECISION_BF16 = 1, SRF_PRECISION_FP16 = 2 };

/* Dynamic loss scale in device memory, with torch.cuda.amp.GradScaler's
 * semantics (torch/amp/grad_scaler.py: init scale 2^16, growth 2 every 2000
 * clean steps, backoff 0.5): the FP16 backward multiplies the incoming
 * gradients by `scale` and its weight/bias gradients by inv_scale, and sets
 * found_inf when a stored 16-bit value is not finite or out of range (the
 * forward sets it too).  A step that found inf is skipped (srf_adam_step's
 * skip_dev) and backs the scale off. */
typedef struct {
    float scale;
    float inv_scale;
    int32_t found_inf;
    int32_t growth_tracker;
} srf_loss_scaler;

/* scaler_dev = {init_scale, 1 / init_scale, 0, 0} (torch.cuda.amp.GradScaler's
 * constructor, torch/amp/grad_scaler.py). */
int srf_loss_scaler_init(srf_loss_scaler* scaler_dev, float init_scale, void* stream);
/* Per-call scale for a backward whose gradients have no running scale (no
 * reference counterpart: the reference trains in FP32): the largest |value| over
 * a (na) and b (nb) maps to within a factor 2 below target, scale =
 * 2^floor(log2(target / max)) in [2^-24, 2^40] (1 when max is 0); found_inf and
 * growth_tracker are cleared. */
int srf_loss_scaler_fit(srf_loss_scaler* scaler_dev, const float* a, int64_t na, const float* b, int64_t nb,
                        float target, void* stream);
/* End of a step: if found_inf, scale *= backoff and growth_tracker = 0, else
 * growth_tracker += 1 and, on reaching growth_interval, scale *= growth and
 * growth_tracker = 0; then inv_scale = 1 / scale and found_inf = 0
 * (torch's _amp_update_scale_). */
int srf_loss_scaler_update(srf_loss_scaler* scaler_dev, float growth, float backoff, int growth_interval,
                           void* stream);

/* Number of parameter tensors and, for index i, the reference state_dict name
 * and element count (order = the order the params/grads arrays use). */
int srf_nerf_mlp_num_params(const srf_nerf_mlp_desc* desc);
int srf_nerf_mlp_param_info(const srf_nerf_mlp_desc* desc, int index, char* name, int name_len, int64_t* numel);

/* Workspace bytes for srf_nerf_mlp_forward (+ backward when for_backward). */
size_t srf_nerf_mlp_workspace_size(const srf_nerf_mlp_desc* desc, int64_t m, int precision, int for_backward);

/* Forward of one MLP over m samples.  pts (m,3); dirs (ceil(m/dir_div),3) per-ray
 * directions shared by dir_div consecutive samples (NULL when !use_view_dirs);
 * sigma_noise (m) pre-scaled raw_noise_std*randn or NULL.  Outputs sigma (m)
 * after ReLU and rgb (m,3) after sigmoid.  With for_backward, the workspace keeps
 * what srf_nerf_mlp_backward needs (same workspace, same inputs).  scaler
 * (optional; 16-bit precisions) receives found_inf when an activation overflows.
 * Replaces MLP.forward (src/models/SimpleNeRF17.py:696-785) including the
 * chunking of run_network/batchify (:419-484). */
int srf_nerf_mlp_forward(const srf_nerf_mlp_desc* desc, const float* const* params, const float* pts,
                         const float* dirs, int dir_div, int64_t m, const float* sigma_noise, float* sigma,
                         float* rgb, int precision, int for_backward, void* workspace, size_t workspace_bytes,
                         srf_loss_scaler* scaler, void* stream);
/* Forward path of the 16-bit NeRF MLP (MLP.forward, SimpleNeRF17.py:696-785, at
 * BF16 / FP16 precision; the switch itself has no reference counterpart): mode 0
 * runs one tcgen05 kernel per layer after the encoder; 1 (default) runs the layers of a
 * forward-only call (for_backward = 0) as one fused kernel that keeps each
 * 128-sample tile's activations in shared memory from the encodings to the
 * heads; 2 also fuses the forward of for_backward calls, which then stores the
 * activations the backward reads from the fused kernel (measured slower than the
 * per-layer kernels).  Layouts the fused kernel does not cover (trunk width other
 * than 256, point PE degree above 10, the points-augmentation variant, a view
 * branch other than one 128-wide layer) always run per layer.  The paths form
 * the same products in the same order and round the same activations; the head
 * dot products sum their partials in another order (last-bit differences).
 * Returns the previous mode (0..2); mode < 0 only queries; a mode above 2 changes
 * nothing and returns -SRF_ERR_SHAPE.  Process-wide setting. */
int srf_nerf_mlp_fused_path(int mode);

/* Backward: dsigma (m) w.r.t. the ReLU'd sigma, drgb (m,3) w.r.t. the sigmoid
 * rgb; dir_div as in the forward.  grads[i] receives (accumulate ? += : =) the
 * gradient of params[i].  Uses the activations the forward left in the workspace.
 * SRF_PRECISION_FP16 requires scaler (the gradients are unscaled before they are
 * written; a non-finite or out-of-range scaled value sets found_inf). */
int srf_nerf_mlp_backward(const srf_nerf_mlp_desc* desc, const float* const* params, const float* dsigma,
                          const float* drgb, int dir_div, int64_t m, float* const* grads, int accumulate,
                          int precision, void* workspace, size_t workspace_bytes, srf_loss_scaler* scaler,
                          void* stream);

/* BF16 tcgen05 dense layer (the building block of the BF16 MLP path):
 * out[m, :n] = relu?(x0[m, :k0] . Wb^T + x1[m, :k1] . Wb'^T + bias) * (mask > 0)?
 * where W (w_rows x ldw, BF16, row-major like nn.Linear.weight) supplies rows
 * [w_row0, w_row0 + n) over columns [0, k0 + k1).  k0, k1 multiples of 64;
 * n in {64, 128, 256}; BF16 pointers 16-byte aligned, leading dims multiples
 * of 8.  colsum (n floats, optional) accumulates the column sums of the output.
 * Replaces one torch.nn.Linear (+ReLU) of MLP.forward (src/models/SimpleNeRF17.py:729-733). */
int srf_bf16_linear(void* out, int64_t ld_out, const void* x0, int64_t ld0, int k0, const void* x1, int64_t ld1,
                    int k1, const void* w, int64_t ldw, int w_rows, int w_row0, const float* bias, int64_t m, int n,
                    int relu, const void* mask, int64_t ld_mask, float* colsum, void* stream);
/* BF16 weight gradient partials: partial[s, j, k] = sum over split s of
 * dz[i, j] * [x0 | x1][i, k]; *splits receives the split count (sum over s
 * gives dW).  n_dz multiple of 128, k0 + k1 <= 512 (multiples of 64).
 * Replaces the autograd weight gradient of those nn.Linear layers. */
size_t srf_bf16_wgrad_workspace_size(int n_dz, int k_total);
int srf_bf16_wgrad(float* partial, size_t partial_bytes, int* splits, const void* dz, int64_t ld_dz, int n_dz,
                   const void* x0, int64_t ld0, int k0, const void* x1, int64_t ld1, int k1, int64_t m,
                   void* stream);

/* ------------------------------------------------------------------------ */
/* Alpha compositing                                                         */
/* ------------------------------------------------------------------------ */

enum {
    SRF_COMPOSITE_NDC = 1,        /* z is NDC depth; also emit depth_ndc / depth_var_ndc  */
    SRF_COMPOSITE_WHITE_BKGD = 2, /* rgb += 1 - acc                                        */
    /* transmittance T_i = exp(-sum_{j<i} sigma_j delta_j) (one exclusive sum scan)
     * instead of the reference's exclusive cumprod of 1 - alpha_j + 1e-10; the two
     * differ by the 1e-10 terms and rounding only.  Rays of at most 256 samples
     * (SRF_ERR_UNSUPPORTED beyond).  The 16-bit training steps use it. */
    SRF_COMPOSITE_EXP_PREFIX = 4
};

typedef struct {
    int n_rays, n_samples, flags;
    float distance_scale;          /* 1 for NeRF, tensor_configs['distance_scale'] for TensoRF */
    const float* sigma;            /* (N,S)                                       */
    const float* rgb;              /* (N,S,3); NULL = zero colours (density pass) */
    const float* z;                /* (N,S) depth used for delta (NDC depth if NDC) */
    const float* rays_d;           /* (N,3) world directions                       */
    const float* rays_o;           /* (N,3) world origins (NDC only)               */
    const float* rays_d_ndc;       /* (N,3) NDC directions (NDC only)              */
    const uint8_t* white_per_ray;  /* (N) optional per-ray white-background flags  */
    /* forward outputs (any may be NULL) */
    float *rgb_map, *acc, *depth, *depth_var, *depth_ndc, *depth_var_ndc, *alpha, *visibility, *weights;
    /* backward inputs: gradients of the outputs (any may be NULL = zero) */
    const float *g_rgb, *g_acc, *g_depth, *g_depth_var, *g_depth_ndc, *g_depth_var_ndc, *g_weights;
    /* backward outputs */
    float *d_sigma, *d_rgb;
} srf_composite_args;

/* Replaces SimpleNeRF.volume_rendering (src/models/SimpleNeRF17.py:486-539),
 * convert_depth_from_ndc (:541-558), LowRankTensor.get_volume_rendering_weights
 * and volume_render (src/models/SimpleTensoRF09.py:767-819). */
int srf_composite_forward(const srf_composite_args* args, void* stream);
/* Adjoint: reverse-scan transmittance gradient, recomputing the forward per ray. */
int srf_composite_backward(const srf_composite_args* args, void* stream);

/* A training loss evaluated inside compositing, so that the loss gradient feeds
 * the compositing adjoint without a round trip of the per-ray outputs or the
 * (N,S) weights through memory:
 *   rgb_weight * mean_rays mean_channels (rgb - target_rgb)^2
 *       (MSE14.compute_mse, src/loss_functions/MSE14.py:81-94; rgb after the white background)
 * + depth_weight / n_depth_rays * sum over depth_mask rays of |depth - target_depth|
 *       (the training step's L1 depth term) or (depth - target_depth)^2 with depth_squared
 *       (SparseDepthMSE14.compute_depth_loss, src/loss_functions/SparseDepthMSE14.py:84-97)
 * + mc_weight / n_mc_rays * sum over mc_mask rays of the binned entropy of the weights
 *       (MassConcentrationLoss06.compute_entropy_loss, src/loss_functions/MassConcentrationLoss06.py:63-83;
 *        num_bins <= 32, 0 = no entropy term).
 * NULL targets / masks: the term is off / every ray counts. */
typedef struct {
    const float* target_rgb;       /* (N,3) or NULL */
    float rgb_weight;
    const float* target_depth;     /* (N) or NULL   */
    const uint8_t* depth_mask;     /* (N) or NULL   */
    int n_depth_rays;
    float depth_weight;
    int depth_squared;
    int num_bins;
    const uint8_t* mc_mask;        /* (N) or NULL   */
    int n_mc_rays;
    float mc_weight;
    float* loss;                   /* device float the forward adds the loss value to */
} srf_composite_loss;
/* srf_composite_forward that also adds the loss value to *loss->loss (the losses
 * of MSE14.py:81-94, MassConcentrationLoss06.py:63-83 and the depth term above,
 * evaluated in the compositing epilogue). */
int srf_composite_forward_loss(const srf_composite_args* args, const srf_composite_loss* loss, void* stream);
/* srf_composite_backward whose output gradients are the loss's (recomputed from the
 * ray's samples; the autograd of the same loss modules) plus any g_* the args carry
 * (e.g. a depth-consistency term, CoarseFineConsistencyLoss33.py:35-44).  Both:
 * rays of at most 256 samples (SRF_ERR_UNSUPPORTED beyond). */
int srf_composite_backward_loss(const srf_composite_args* args, const srf_composite_loss* loss, void* stream);

/* out (N,C) = sum_s weights (N,S) * values (N,S,C), C <= 4, and its adjoint.
 * Replaces LowRankTensor.volume_render (src/models/SimpleTensoRF09.py:816-819). */
int srf_weighted_sum(const float* weights, const float* values, int n_rays, int n_samples, int channels, float* out,
                     void* stream);
int srf_weighted_sum_backward(const float* weights, const float* values, const float* g_out, int n_rays,
                              int n_samples, int channels, float* d_weights, float* d_values, void* stream);

/* ------------------------------------------------------------------------ */
/* TensoRF VM decomposition                                                  */
/* ------------------------------------------------------------------------ */

typedef struct {
    int res[3];            /* grid resolution per world axis (x, y, z)                    */
    int n_comp[3];         /* components per plane/line pair i (matrix_axes[i], vector_axes[i]) */
    float* planes[3];      /* plane i: logical (1,R_i,res[m1],res[m0]), channels-last (H,W,R_i) */
    float* lines[3];       /* line i:  logical (1,R_i,res[v],1), channels-last (L,R_i)         */
} srf_vm_grid;

/* Density features: out[p] = sum_i sum_r plane_i[r](x_m0,x_m1) * line_i[r](x_v) at
 * normalised points pts (P,3) (bilinear, align_corners=True, zero padding).
 * Replaces VmDecomposedTensor.get_volume_density (src/models/SimpleTensoRF09.py:1214-1239). */
int srf_vm_density_forward(const srf_vm_grid* grid, const float* pts, int64_t n_pts, float* features,
                           void* stream);
/* Adds d(features) into the grid gradients (grad_grid: same layout as grid). */
int srf_vm_density_backward(const srf_vm_grid* grad_grid, const srf_vm_grid* grid, const float* pts,
                            int64_t n_pts, const float* d_features, void* stream);
/* Colour features (P, sum R_i): concat_i plane_i * line_i.
 * Replaces VmDecomposedTensor.get_color lookups (src/models/SimpleTensoRF09.py:1252-1262). */
int srf_vm_color_forward(const srf_vm_grid* grid, const float* pts, int64_t n_pts, float* features,
                         void* stream);
int srf_vm_color_backward(const srf_vm_grid* grad_grid, const srf_vm_grid* grid, const float* pts,
                          int64_t n_pts, const float* d_features, void* stream);
/* Deterministic forms of the two adjoints: the scatter-add's FP32 atomics sum in
 * an order that varies from run to run; these round every contribution once to a
 * 64-bit fixed-point integer (a power-of-two scale S from the largest |d_features|
 * and |grid value| and the point count, so that no partial sum leaves 63 bits),
 * add them with integer atomics, whose sums are independent of order, and add
 * acc / S into grad_grid: bitwise reproducible, each contribution exact to
 * n max|d| max|grid| 2^-63.  workspace: srf_vm_backward_fixed_workspace_size(grid)
 * bytes, 16-byte aligned (one int64 per grid element). */
size_t srf_vm_backward_fixed_workspace_size(const srf_vm_grid* grid);
int srf_vm_density_backward_fixed(const srf_vm_grid* grad_grid, const srf_vm_grid* grid, const float* pts,
                                  int64_t n_pts, const float* d_features, void* workspace, size_t workspace_bytes,
                                  void* stream);
int srf_vm_color_backward_fixed(const srf_vm_grid* grad_grid, const srf_vm_grid* grid, const float* pts,
                                int64_t n_pts, const float* d_features, void* workspace, size_t workspace_bytes,
                                void* stream);

/* CP decomposition (CpDecomposedTensor, src/models/SimpleTensoRF09.py:964-1123): only
 * grid->lines are used (planes ignored), line i along world axis vector_axes[i] =
 * (2, 1, 0)[i], channels-last (L_i, R) with the same R for all three.  Density
 * features out[p] = sum_r prod_i line_i[r] (:1070-1080); colour features (P, R):
 * prod_i line_i[r] (:1091-1098).  The backward adds into grad_grid's lines. */
int srf_cp_density_forward(const srf_vm_grid* grid, const float* pts, int64_t n_pts, float* features, void* stream);
int srf_cp_density_backward(const srf_vm_grid* grad_grid, const srf_vm_grid* grid, const float* pts, int64_t n_pts,
                            const float* d_features, void* stream);
int srf_cp_color_forward(const srf_vm_grid* grid, const float* pts, int64_t n_pts, float* features, void* stream);
int srf_cp_color_backward(const srf_vm_grid* grad_grid, const srf_vm_grid* grid, const float* pts, int64_t n_pts,
                          const float* d_features, void* stream);

/* Sample validity for TensoRF: inside the bbox and (when alpha_volume != NULL)
 * alpha-mask trilinear value > 0; writes normalised points and a 0/1 mask.
 * Replaces LowRankTensor.forward:705-710 + AlphaGridMask.sample_alpha
 * (src/models/SimpleTensoRF09.py:1342-1349) + normalize_points (:763-765). */
int srf_tensorf_sample_mask(const float* rays_o, const float* rays_d, const float* z, int n_rays, int n_samples,
                            const float* bbox /* host (2,3) */, const float* alpha_volume, int vol_d, int vol_h,
                            int vol_w, const float* alpha_bbox /* host (2,3) */, float* pts_norm,
                            uint8_t* mask, void* stream);
/* Alpha-mask query alone: out[p] = (trilinear(volume, pts_norm[p]) > 0)
 * (AlphaGridMask.sample_alpha, src/models/SimpleTensoRF09.py:1342-1349). */
int srf_alpha_mask_query(const float* alpha_volume, int vol_d, int vol_h, int vol_w, const float* pts_norm,
                         int64_t n_pts, uint8_t* out, void* stream);

/* ------------------------------------------------------------------------ */
/* Grid maintenance (planes (H,W,R) and lines (L,1,R) channels-last)          */
/* ------------------------------------------------------------------------ */

/* Dense alpha on the nodes of the grid's res[0] x res[1] x res[2] lattice:
 * node (x,y,z) at bbox_lo (1 - s) + bbox_hi s with s = torch.linspace(0,1,res)
 * per axis; alpha = clamp(1 - exp(-sigma step), 0, 1), sigma the activated VM
 * density (density_mode 0 ReLU, 1 softplus(x + offset)), 0 where the optional
 * current alpha mask (volume + box as in srf_tensorf_sample_mask) is empty.
 * alpha is written z-major, (res[2], res[1], res[0]).  bbox, alpha_bbox: host (2,3).
 * Replaces LowRankTensor.update_alpha_mask's dense pass and compute_alpha
 * (src/models/SimpleTensoRF09.py:849-858, 878-897). */
int srf_vm_alpha_grid(const srf_vm_grid* grid, const float* bbox, const float* alpha_volume, int vol_d, int vol_h,
                      int vol_w, const float* alpha_bbox, float step, int density_mode, float density_offset,
                      float* alpha, void* stream);
/* 3x3x3 max-pool (padding 1, stride 1) of alpha (gz, gy, gx) and threshold
 * (>= threshold -> 1, else 0) into volume (gz, gy, gx); bounds (6 device ints)
 * receive (gx-1-min x, gy-1-min y, gz-1-min z, max x, max y, max z) over the
 * occupied nodes, all -1 when none is occupied.
 * Replaces SimpleTensoRF09.py:859-874 (max_pool3d, threshold, occupied box). */
int srf_alpha_pool_threshold(const float* alpha, int gx, int gy, int gz, float threshold, float* volume,
                             int32_t* bounds, void* stream);
/* Bilinear resampling with align_corners=True of a channels-last (h, w, comps)
 * plane (or a (h, 1, comps) line) to (h_new, w_new, comps).
 * Replaces F.interpolate in upsample_vectors_and_matrices (SimpleTensoRF09.py:1284-1301). */
int srf_resample_grid(const float* src, int h, int w, int comps, float* dst, int h_new, int w_new, void* stream);
/* Crop rows [row0, row0 + h_new) x columns [col0, col0 + w_new) of a channels-last
 * (h, w, comps) plane or line into dst (h_new, w_new, comps).
 * Replaces the slicing of shrink_tensor (SimpleTensoRF09.py:1303-1320). */
int srf_crop_grid(const float* src, int h, int w, int comps, int row0, int col0, float* dst, int h_new, int w_new,
                  void* stream);

/* Stream compaction: idx[0..count) = positions where mask != 0 (ascending).
 * count is written to *count_dev (device int).  Workspace: srf_compact_workspace_size. */
size_t srf_compact_workspace_size(int64_t n);
int srf_compact(const uint8_t* mask, int64_t n, int32_t* idx, int32_t* count_dev, void* workspace,
                size_t workspace_bytes, void* stream);
/* Stream compaction for callers that cannot allocate device memory (no
 * counterpart in the reference; the reference compacts with torch boolean
 * indexing).  Same result as srf_compact, but it takes no workspace: its scratch
 * is a fixed 64 KB array inside the library, present on every GPU that loads it
 * until the process exits.  Meant for code that runs inside another framework's
 * fixed memory pool, under a no-allocation guarantee, or behind a binding that
 * only holds the mask and output pointers.
 *   - n may not exceed SRF_COMPACT_NOALLOC_MAX_ELEMENTS; larger masks return
 *     SRF_ERR_SHAPE without launching anything (use srf_compact for those).
 *   - The first call on a device looks up the array's device address; make that
 *     first call before any CUDA stream capture on that device.  The address is
 *     cached per device for the context it was looked up in: after
 *     cudaDeviceReset, reload the library before calling again.
 *   - All calls share the one array: calls whose kernels may overlap on the GPU
 *     (different streams, or different host threads) race and must be ordered by
 *     the caller.  Each call fully rewrites the scratch it reads. */
#define SRF_COMPACT_NOALLOC_MAX_BLOCKS 16384
#define SRF_COMPACT_NOALLOC_MAX_ELEMENTS (SRF_COMPACT_NOALLOC_MAX_BLOCKS * 1024)
int srf_compact_noalloc(const uint8_t* mask, int64_t n, int32_t* idx, int32_t* count_dev, void* stream);

/* Mask of weights > threshold (surface samples, src/models/SimpleTensoRF09.py:726). */
int srf_threshold_mask(const float* x, int64_t n, float threshold, uint8_t* mask, void* stream);

/* Gather rows src[idx[i]] -> dst[i] (cols floats each), for i < *count_dev (max n). */
int srf_gather_rows(float* dst, const float* src, int64_t src_rows, const int32_t* idx, const int32_t* count_dev,
                    int64_t n, int cols, int src_row_div, void* stream);
/* Scatter rows src[i] -> dst[idx[i]] (dst not cleared; rows not in idx untouched). */
int srf_scatter_rows(float* dst, int64_t dst_rows, const float* src, const int32_t* idx, const int32_t* count_dev,
                     int64_t n, int cols, void* stream);

/* Density activation on compacted features: ReLU (mode 0) or softplus(x+offset)
 * (mode 1), written to sigma[idx[i]] of the rows-long dense sigma; backward
 * multiplies by the derivative.
 * Replaces LowRankTensor.get_density_predictor (src/models/SimpleTensoRF09.py:671-679).
 * The row functions above take the row count of the dense side: an index outside
 * [0, rows) (or past src_rows after the division) is skipped and sets the range
 * bit of the device flag (srf_read_device_flag) instead of touching memory. */
int srf_density_activation(float* sigma_dense, int64_t rows, const float* features, const int32_t* idx,
                           const int32_t* count_dev, int64_t n, int mode, float offset, void* stream);
int srf_density_activation_backward(float* d_features, const float* d_sigma_dense, int64_t rows,
                                    const float* features, const int32_t* idx, const int32_t* count_dev, int64_t n,
                                    int mode, float offset, void* stream);

/* ------------------------------------------------------------------------ */
/* Generic dense layer (TensoRF renderer MLP and basis matrix)               */
/* ------------------------------------------------------------------------ */

enum { SRF_ACT_NONE = 0, SRF_ACT_RELU = 1, SRF_ACT_SIGMOID = 2 };

/* y[r, :n] = act(x[r, :k] . W^T + bias) for r < rows (rows = *rows_dev if rows_dev
 * else max_rows).  W (n,k) row-major as torch.nn.Linear.weight; bias may be NULL.
 * Replaces the nn.Linear layers of MlpFeaturesColorPredictor and
 * basis_matrix_color (src/models/SimpleTensoRF09.py:1151,1389-1392). */
int srf_linear_forward(float* y, int ldy, const float* x, int ldx, const float* weight, const float* bias,
                       int64_t max_rows, const int32_t* rows_dev, int n, int k, int act, void* stream);
/* dx = (dy * act'(y)) . W ; dW (+)= dz^T x ; db (+)= sum dz, where dz = dy*act'(y).
 * Any of dx, dw, db may be NULL; y may be NULL when act is SRF_ACT_NONE.  dz scratch
 * (rows, n) is caller-provided (may alias dy). */
int srf_linear_backward(float* dx, int lddx, float* dw, float* db, const float* dy, int lddy, const float* y,
                        int ldy, const float* x, int ldx, const float* weight, float* dz_scratch,
                        int64_t max_rows, const int32_t* rows_dev, int n, int k, int act, int accumulate,
                        void* stream);
/* TensoRF renderer on tcgen05 tensor cores (16-bit operands, FP32 accumulation):
 * basis_matrix_color (n_comp -> features, no bias) followed by
 * MlpFeaturesColorPredictor: x = [PE(features, Lf), PE(view, Lv)] -> units ReLU
 * -> units ReLU -> 3 sigmoid.  Replaces SimpleTensoRF09.py:1151 and :1370-1421
 * for precision SRF_PRECISION_BF16 / SRF_PRECISION_FP16 (the FP32 path is
 * srf_linear_* + srf_positional_encoding).  units must be 128 or 256.
 * params / grads: {basis (features x n_comp), W1 (units x k1), b1, W2 (units x units),
 * b2, W3 (3 x units), b3}, k1 = features (2 Lf + 1) + 3 (2 Lv + 1); grads accumulate.
 * view_dirs (m,3) per sample.  The backward writes d_feats (m, n_comp) and needs
 * the forward's workspace (for_backward) and, for FP16, a loss scaler. */
typedef struct {
    int n_comp;               /* colour components: sum of the three planes' R */
    int features;             /* features_dimension_color                      */
    int units;                /* num_units_color_predictor                     */
    int features_pe_degree;
    int views_pe_degree;
    int view_dependent;       /* view_dependent_color (view PE appended)       */
} srf_tensorf_renderer_desc;

/* Workspace bytes of the renderer forward (+ backward); no reference counterpart. */
size_t srf_tensorf_renderer_workspace_size(const srf_tensorf_renderer_desc* desc, int64_t m, int precision,
                                           int for_backward);
/* Forward / backward of the renderer above (SimpleTensoRF09.py:1151, :1370-1421 and
 * their autograd). */
int srf_tensorf_renderer_forward(const srf_tensorf_renderer_desc* desc, const float* const* params, const float* feats,
                                 const float* view_dirs, int64_t m, float* rgb, int precision, int for_backward,
                                 void* workspace, size_t workspace_bytes, srf_loss_scaler* scaler, void* stream);
int srf_tensorf_renderer_backward(const srf_tensorf_renderer_desc* desc, const float* const* params,
                                  const float* feats, const float* d_rgb, int64_t m, float* const* grads,
                                  float* d_feats, int precision, void* workspace, size_t workspace_bytes,
                                  srf_loss_scaler* scaler, void* stream);
/* No reference counterpart.  The basis adjoint of the 16-bit renderer backward
 * (d_feats = dB . Wb, dWb += dB^T feats, dB from the PE adjoint): tensor_cores = 1
 * (default) takes the TF32 tcgen05 pass plus a dWb reduction where the shapes fit
 * (C a multiple of 16 up to 256), 0 always the fused FP32 SIMT pass.  Both give the
 * same gradients up to the TF32 rounding of dB and Wb in d_feats.  Process-wide
 * setting. */
int srf_tensorf_basis_adjoint_path(int tensor_cores);
/* Positional-encoding backward d x (m,dims) from d out (m, ld): the autograd of
 * the TensoRF colour predictor's feature PE (MlpFeaturesColorPredictor,
 * SimpleTensoRF09.py:1370-1421, the encoding of SimpleNeRF17.py:581-613). */
int srf_positional_encoding_backward(float* dx, const float* x, const float* dout, int ld_dout, int64_t m,
                                     const int32_t* rows_dev, int dims, int degree, void* stream);

/* ------------------------------------------------------------------------ */
/* Training-step helpers                                                     */
/* ------------------------------------------------------------------------ */

/* The training step's loss on one net's outputs: mean over rays of mean over channels
 * of (rgb - target)^2 (MSE14.compute_mse, src/loss_functions/MSE14.py:81-94) plus
 * depth_weight * mean |depth - target_depth| over rays with depth_mask != 0.
 * Adds the loss to *loss_dev (device float) and writes g_rgb (N,3), g_depth (N). */
int srf_rgb_depth_loss(const float* rgb, const float* target_rgb, const float* depth, const float* target_depth,
                       const uint8_t* depth_mask, int n_rays, int n_depth_rays, float depth_weight,
                       float* loss_dev, float* g_rgb, float* g_depth, void* stream);

/* Fused Adam (torch.optim.Adam semantics, bias-corrected, no amsgrad) over n
 * elements; step is the 1-based step count after this update, or, when
 * step_dev != NULL, read from device memory (for CUDA-graph replays).  When
 * skip_dev != NULL and *skip_dev != 0 nothing is updated (a loss-scaled step
 * that found inf, as GradScaler.step skips optimizer.step).
 * Replaces the optimizer step of Trainer10.train_one_iter (src/Trainer10.py:110). */
int srf_adam_step(float* param, const float* grad, float* exp_avg, float* exp_avg_sq, int64_t n, float lr,
                  float beta1, float beta2, float eps, float weight_decay, int step, const int32_t* step_dev,
                  const int32_t* skip_dev, void* stream);
/* One tensor of a multi-tensor Adam step (its own learning rate, as one param
 * group of torch.optim.Adam). */
typedef struct srf_adam_tensor {
    float* param;
    const float* grad;
    float* exp_avg;
    float* exp_avg_sq;
    int64_t n;
    float lr;
} srf_adam_tensor;
/* srf_adam_step over several tensors with one launch per 64 tensors (the same
 * per-element arithmetic); tensors with n == 0 are skipped.  Replaces the
 * optimizer step over a model's param groups (Trainer10.py:110,
 * SimpleTensoRF09.py:1167-1194 groups). */
int srf_adam_multi_step(const srf_adam_tensor* tensors, int n_tensors, float beta1, float beta2, float eps,
                        float weight_decay, int step, const int32_t* step_dev, const int32_t* skip_dev, void* stream);
/* Squared depth error with the matching gradients (accumulated into grad_pred and
 * grad_target, either may be NULL): with m_r = mask[r] (all ones when mask == NULL)
 * and count = n, or the number of masked rays when mean_over_mask,
 *   loss += weight * sum_r m_r (pred_r - target_r)^2 / count,
 *   grad_pred[r] += 2 weight m_r (pred_r - target_r) / count, grad_target[r] -= the same.
 * Replaces AugmentationsDepthLoss11.compute_depth_mse
 * (src/loss_functions/AugmentationsDepthLoss11.py:208-226: count = n, target detached:
 * grad_target NULL; the reprojection mask of :105-190 is the caller's),
 * SparseDepthMSE14.compute_depth_loss (src/loss_functions/SparseDepthMSE14.py:84-97:
 * mean_over_mask) and CoarseFineConsistencyLoss33 (src/loss_functions/
 * CoarseFineConsistencyLoss33.py:35-44: no mask, gradients into both). */
int srf_depth_mse_loss(const float* pred, const float* target, const uint8_t* mask, int n, float weight,
                       int mean_over_mask, float* loss_dev, float* grad_pred, float* grad_target, void* stream);
/* MassConcentrationLoss06.compute_entropy_loss
 * (src/loss_functions/MassConcentrationLoss06.py:63-83): weights (n_rays, n_samples)
 * summed over num_bins contiguous bins (n_samples / num_bins samples each, one more
 * in the bins torch.linspace(0, num_bins - 1, n_samples % num_bins).long() picks),
 * loss += weight * mean over masked rays of sum_bins -(b + 1e-3) ln(b + 1e-3), and
 * grad_weights (may be NULL) += its gradient (feed it to srf_composite_backward's
 * g_weights).  num_bins in [1, 64]. */
int srf_mass_concentration_loss(const float* weights, int n_rays, int n_samples, int num_bins, const uint8_t* mask,
                                float weight, float* loss_dev, float* grad_weights, void* stream);
/* The masks of AugmentationsDepthLoss11.compute_loss_nerf
 * (src/loss_functions/AugmentationsDepthLoss11.py:105-190) for n_rays NeRF rays:
 * per ray, the camera b with the nearest origin to the ray's own camera (ties: the
 * lowest index), the points o + d depth1 and o + d depth2 reprojected into b with
 * the first view's intrinsics (CommonUtils04.reproject, src/utils/CommonUtils04.py:227-253)
 * and rounded, and the patch_h x patch_w RMSE of the ray's own patch against the
 * patch at each reprojection (zero outside the image).  mask1 = depth1 is the more
 * consistent one (a target for depth2), mask2 the reverse, with the reference's
 * validity and tie rules.  pixel_ids (n,3) int32 (image, x, y); poses (n_views,4,4)
 * camera-to-world; intrinsics0 (3,3); images (n_views, height, width, channels).
 * The reference then adds compute_depth_mse(depth1, depth2, mask2) (srf_depth_mse_loss
 * with grad_target NULL); its second term, on mask1, sees tensors the first zeroed
 * in place outside mask2 and so contributes only on mask1 & mask2, which is empty. */
int srf_depth_reprojection_masks(const float* rays_o, const float* rays_d, const float* depth1, const float* depth2,
                                 const int32_t* pixel_ids, int n_rays, const float* poses, int n_views,
                                 const float* intrinsics0, const float* images, int height, int width, int channels,
                                 int patch_w, int patch_h, float rmse_threshold, uint8_t* mask1, uint8_t* mask2,
                                 void* stream);
/* The same masks for CoarseFineConsistencyLoss34.compute_loss_nerf
 * (src/loss_functions/CoarseFineConsistencyLoss34.py:89-168): depth1 the main coarse
 * depth, depth2 the main fine depth, and no rule for rays whose two reprojections
 * both leave the image (AugmentationsDepthLoss11's :176-181 is absent there).  The
 * loss is then compute_depth_mse(depth_coarse, depth_fine, mask2) as above, and on
 * sparse-depth rays compute_loss_sd (:170-187): srf_depth_mse_loss of the coarse
 * depth against the detached fine depth over those rays. */
int srf_coarse_fine_reprojection_masks(const float* rays_o, const float* rays_d, const float* depth_coarse,
                                       const float* depth_fine, const int32_t* pixel_ids, int n_rays,
                                       const float* poses, int n_views, const float* intrinsics0, const float* images,
                                       int height, int width, int channels, int patch_w, int patch_h,
                                       float rmse_threshold, uint8_t* mask1, uint8_t* mask2, void* stream);
/* One grid of the total-variation loss: element (c, h, w) of the (1, channels,
 * height, width) parameter at data[c*stride_channel + h*stride_height +
 * w*stride_width] (channels-last: stride_channel 1); grad (may be NULL) has the
 * same strides. */
typedef struct srf_tv_component {
    const float* data;
    float* grad;
    int channels, height, width;
    int64_t stride_channel, stride_height, stride_width;
} srf_tv_component;
/* TotalVariationLoss04.compute_tv_loss (src/loss_functions/TotalVariationLoss04.py:97-116)
 * over up to 8 components (a VM model's three planes, or a CP model's three lines):
 * loss_dev (may be NULL) += weight * sum_i 2 (sum (P[h+1] - P[h])^2 / numel_h +
 * sum (P[w+1] - P[w])^2 / numel_w), numel_* the element counts of the difference
 * tensors floored at 1; each component's grad += s * d loss / d data, s =
 * *scale_dev, or 1 when scale_dev is NULL (a device scalar, e.g. autograd's
 * incoming gradient).  weight = iter_weight * the loss's weight_density or
 * weight_color. */
int srf_tv_loss(const srf_tv_component* components, int n_components, float weight, const float* scale_dev,
                float* loss_dev, void* stream);
/* Online tuning of equivalent kernel shapes (on by default).  The first call of a
 * tuned launch site with a new shape times each candidate on that call's own
 * inputs and caches the fastest: the layer GEMM's epilogue warp count (site 1, key
 * BN, K blocks, epilogue flags), the TensoRF basis pass's tile (site 2, key C, k1p)
 * and the VM colour gather's lanes per point (site 3, key R0, R1, R2).  Nothing is
 * timed during CUDA-graph capture or when disabled (the launches then take the
 * built-in rules), and only launches whose outputs are plain overwrites are tuned.
 * The table can be listed (count / entry) and preloaded (set) to reuse choices. */
int srf_autotune_enable(int on);
int srf_autotune_count(void);
int srf_autotune_entry(int index, int* site, int64_t* a, int64_t* b, int64_t* c, int* choice);
int srf_autotune_set(int site, int64_t a, int64_t b, int64_t c, int choice);
int srf_autotune_clear(void);
/* *counter_dev += value on the stream (advances a graph-replayed step count),
 * unless skip_dev != NULL and *skip_dev != 0. */
int srf_counter_add(int32_t* counter_dev, int value, const int32_t* skip_dev, void* stream);

/* Device-side batch assembly for cached-ray training (replaces
 * DataPreprocessor10.select_batch_indices and load_nerf_cached_batch,
 * src/data_preprocessors/DataPreprocessor10.py:496-549, whose host numpy shuffle and
 * copies keep the training iteration out of a CUDA graph).  Batch b (read from
 * *batch_counter_dev; 0 when NULL) takes rays ((b mod B) n_rays + i) of epoch
 * (b div B)'s order, B = pool_size div n_rays; each epoch's order is a fresh keyed
 * random permutation of [0, pool_size) (seed, epoch), so every epoch visits
 * B n_rays distinct rays (the pool_size mod n_rays rays an epoch leaves over are
 * the ones the reference's shorter last slice would take).  Gathers, per batch ray
 * i: out_index[i] (optional), the pool row's pixel id (image, x, y) (optional),
 * its `channels` floats of pool_values (e.g. the target colour), and the camera
 * of its image from intrinsics (n_views,3,3) / extrinsics (n_views,4,4)
 * (optional: per-ray copies for srf_pixel_rays).  With pool_rows (pool_size
 * int32, optional) the permuted positions index that list and the gathers read
 * row pool_rows[...] (the sparse-depth pixels, a subset of the cached rays);
 * table_rows is the row count of pool_pixel_id / pool_values (>= pool_size without
 * pool_rows): a pool_rows entry outside it gathers row 0 and sets the device flag.
 * Advance the counter with srf_counter_add after the step.  pool_size <= 2^30. */
int srf_batch_assemble(const int32_t* pool_rows, const int32_t* pool_pixel_id, const float* pool_values, int channels,
                       int64_t pool_size, int64_t table_rows, int n_rays, uint64_t seed,
                       const int32_t* batch_counter_dev,
                       const float* intrinsics,
                       const float* extrinsics, int n_views, int32_t* out_pixel_id, float* out_values,
                       int32_t* out_index, float* out_intrinsics, float* out_extrinsics, void* stream);
/* n uniforms in [0, 1) from a counter-based hash of (seed, *counter_dev, stream_id,
 * i): the stratified and inverse-CDF uniforms of a captured step
 * (torch.rand at src/models/SimpleNeRF17.py:355, 397), fresh on every replay as the
 * counter advances. */
int srf_uniforms(float* u, int64_t n, uint64_t seed, const int32_t* counter_dev, int stream_id, void* stream);
/* Sample points pts (N*S,3) = o + d * z (src/models/SimpleNeRF17.py:213-215). */
int srf_ray_points(const float* rays_o, const float* rays_d, const float* z, int n_rays, int n_samples, float* pts,
                   void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SRF_GB300_H */
