"""ctypes binding of the srf_gb300 C ABI (``include/srf_gb300.h``).

This is the same binding a Simple-RF maintainer would add on the reference
side: plain pointers, sizes and a CUDA stream cross the boundary; a non-zero
status becomes a ``RuntimeError``.  There is no fallback: if the shared library
is missing, importing the package's kernels raises.
"""
import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, 'libsrf_gb300.so')

c_int, c_float, c_void_p, c_size_t = ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_size_t
c_int64, c_char_p = ctypes.c_int64, ctypes.c_char_p
P = ctypes.c_void_p            # device pointer
FP = ctypes.POINTER(ctypes.c_float)


class NerfMlpDesc(ctypes.Structure):
    _fields_ = [('points_net_depth', c_int), ('points_net_width', c_int), ('views_net_depth', c_int),
                ('views_net_width', c_int), ('points_pe_degree', c_int), ('views_pe_degree', c_int),
                ('points_sigma_pe_degree', c_int), ('use_view_dirs', c_int), ('view_dependent_rgb', c_int),
                ('skip_layer', c_int)]


class CompositeArgs(ctypes.Structure):
    _fields_ = [('n_rays', c_int), ('n_samples', c_int), ('flags', c_int), ('distance_scale', c_float),
                ('sigma', P), ('rgb', P), ('z', P), ('rays_d', P), ('rays_o', P), ('rays_d_ndc', P),
                ('white_per_ray', P),
                ('rgb_map', P), ('acc', P), ('depth', P), ('depth_var', P), ('depth_ndc', P), ('depth_var_ndc', P),
                ('alpha', P), ('visibility', P), ('weights', P),
                ('g_rgb', P), ('g_acc', P), ('g_depth', P), ('g_depth_var', P), ('g_depth_ndc', P),
                ('g_depth_var_ndc', P), ('g_weights', P),
                ('d_sigma', P), ('d_rgb', P)]


class CompositeLoss(ctypes.Structure):
    _fields_ = [('target_rgb', P), ('rgb_weight', c_float), ('target_depth', P), ('depth_mask', P),
                ('n_depth_rays', c_int), ('depth_weight', c_float), ('depth_squared', c_int), ('num_bins', c_int),
                ('mc_mask', P), ('n_mc_rays', c_int), ('mc_weight', c_float), ('loss', P)]


class RendererDesc(ctypes.Structure):
    _fields_ = [('n_comp', c_int), ('features', c_int), ('units', c_int), ('features_pe_degree', c_int),
                ('views_pe_degree', c_int), ('view_dependent', c_int)]


class VmGrid(ctypes.Structure):
    _fields_ = [('res', c_int * 3), ('n_comp', c_int * 3), ('planes', P * 3), ('lines', P * 3)]


class TvComponent(ctypes.Structure):
    _fields_ = [('data', P), ('grad', P), ('channels', c_int), ('height', c_int), ('width', c_int),
                ('stride_channel', c_int64), ('stride_height', c_int64), ('stride_width', c_int64)]


class AdamTensor(ctypes.Structure):
    _fields_ = [('param', P), ('grad', P), ('exp_avg', P), ('exp_avg_sq', P), ('n', c_int64), ('lr', c_float)]


SRF_OK, SRF_ERR_NULL, SRF_ERR_SHAPE, SRF_ERR_ALIGN, SRF_ERR_WORKSPACE, SRF_ERR_CUDA = 0, 1, 2, 3, 4, 5
SRF_ERR_TIMEOUT, SRF_ERR_RANGE, SRF_ERR_UNSUPPORTED = 6, 7, 8
SRF_COMPOSITE_NDC = 1
SRF_COMPOSITE_WHITE_BKGD = 2
SRF_COMPOSITE_EXP_PREFIX = 4
SRF_PRECISION_FP32 = 0
SRF_PRECISION_BF16 = 1
SRF_PRECISION_FP16 = 2
PRECISIONS = {'fp32': SRF_PRECISION_FP32, 'bf16': SRF_PRECISION_BF16, 'fp16': SRF_PRECISION_FP16}
SRF_ACT_NONE, SRF_ACT_RELU, SRF_ACT_SIGMOID = 0, 1, 2

# name -> (restype, argtypes)
_SIGS = {
    'srf_status_string': (c_char_p, [c_int]),
    'srf_version': (c_char_p, []),
    'srf_last_cuda_error': (c_char_p, []),
    'srf_read_device_flag': (c_int, [ctypes.POINTER(c_int), P]),
    'srf_stream_create': (c_int, [ctypes.POINTER(P)]),
    'srf_read_probe_blocks': (c_int, []),
    'srf_read_probe': (c_int, [P, c_int64, c_int, P, P]),
    'srf_stream_destroy': (c_int, [P]),
    'srf_pixel_rays': (c_int, [P, P, P, c_int, c_int, P, P, P]),
    'srf_ndc_rays': (c_int, [P, P, P, P, c_int, c_int, c_int, c_float, P, P, P, P]),
    'srf_stratified_z': (c_int, [P, P, c_int, c_int, c_float, c_float, c_int, P]),
    'srf_sample_pdf': (c_int, [P, P, P, P, c_int, c_int, c_int, P]),
    'srf_fine_z': (c_int, [P, P, P, P, c_int, c_int, c_int, P]),
    'srf_aabb_z': (c_int, [P, P, P, P, c_int, c_int, FP, c_float, c_float, c_float, P]),
    'srf_positional_encoding': (c_int, [P, c_int, P, c_int64, c_int, c_int, P]),
    'srf_nerf_mlp_num_params': (c_int, [ctypes.POINTER(NerfMlpDesc)]),
    'srf_nerf_mlp_param_info': (c_int, [ctypes.POINTER(NerfMlpDesc), c_int, c_char_p, c_int,
                                        ctypes.POINTER(c_int64)]),
    'srf_nerf_mlp_workspace_size': (c_size_t, [ctypes.POINTER(NerfMlpDesc), c_int64, c_int, c_int]),
    'srf_nerf_mlp_forward': (c_int, [ctypes.POINTER(NerfMlpDesc), ctypes.POINTER(P), P, P, c_int, c_int64, P, P, P,
                                     c_int, c_int, P, c_size_t, P, P]),
    'srf_nerf_mlp_backward': (c_int, [ctypes.POINTER(NerfMlpDesc), ctypes.POINTER(P), P, P, c_int, c_int64,
                                      ctypes.POINTER(P), c_int, c_int, P, c_size_t, P, P]),
    'srf_loss_scaler_init': (c_int, [P, c_float, P]),
    'srf_loss_scaler_update': (c_int, [P, c_float, c_float, c_int, P]),
    'srf_loss_scaler_fit': (c_int, [P, P, c_int64, P, c_int64, c_float, P]),
    'srf_bf16_linear': (c_int, [P, c_int64, P, c_int64, c_int, P, c_int64, c_int, P, c_int64, c_int, c_int, P,
                                c_int64, c_int, c_int, P, c_int64, P, P]),
    'srf_bf16_wgrad_workspace_size': (c_size_t, [c_int, c_int]),
    'srf_bf16_wgrad': (c_int, [P, c_size_t, ctypes.POINTER(c_int), P, c_int64, c_int, P, c_int64, c_int, P, c_int64,
                               c_int, c_int64, P]),
    'srf_composite_forward': (c_int, [ctypes.POINTER(CompositeArgs), P]),
    'srf_composite_backward': (c_int, [ctypes.POINTER(CompositeArgs), P]),
    'srf_composite_forward_loss': (c_int, [ctypes.POINTER(CompositeArgs), ctypes.POINTER(CompositeLoss), P]),
    'srf_composite_backward_loss': (c_int, [ctypes.POINTER(CompositeArgs), ctypes.POINTER(CompositeLoss), P]),
    'srf_weighted_sum': (c_int, [P, P, c_int, c_int, c_int, P, P]),
    'srf_weighted_sum_backward': (c_int, [P, P, P, c_int, c_int, c_int, P, P, P]),
    'srf_vm_density_forward': (c_int, [ctypes.POINTER(VmGrid), P, c_int64, P, P]),
    'srf_vm_density_backward': (c_int, [ctypes.POINTER(VmGrid), ctypes.POINTER(VmGrid), P, c_int64, P, P]),
    'srf_vm_color_forward': (c_int, [ctypes.POINTER(VmGrid), P, c_int64, P, P]),
    'srf_vm_color_backward': (c_int, [ctypes.POINTER(VmGrid), ctypes.POINTER(VmGrid), P, c_int64, P, P]),
    'srf_vm_backward_fixed_workspace_size': (ctypes.c_size_t, [ctypes.POINTER(VmGrid)]),
    'srf_vm_density_backward_fixed': (c_int, [ctypes.POINTER(VmGrid), ctypes.POINTER(VmGrid), P, c_int64, P, P,
                                              ctypes.c_size_t, P]),
    'srf_vm_color_backward_fixed': (c_int, [ctypes.POINTER(VmGrid), ctypes.POINTER(VmGrid), P, c_int64, P, P,
                                            ctypes.c_size_t, P]),
    'srf_cp_density_forward': (c_int, [ctypes.POINTER(VmGrid), P, c_int64, P, P]),
    'srf_cp_density_backward': (c_int, [ctypes.POINTER(VmGrid), ctypes.POINTER(VmGrid), P, c_int64, P, P]),
    'srf_cp_color_forward': (c_int, [ctypes.POINTER(VmGrid), P, c_int64, P, P]),
    'srf_cp_color_backward': (c_int, [ctypes.POINTER(VmGrid), ctypes.POINTER(VmGrid), P, c_int64, P, P]),
    'srf_tensorf_sample_mask': (c_int, [P, P, P, c_int, c_int, FP, P, c_int, c_int, c_int, FP, P, P, P]),
    'srf_alpha_mask_query': (c_int, [P, c_int, c_int, c_int, P, c_int64, P, P]),
    'srf_vm_alpha_grid': (c_int, [ctypes.POINTER(VmGrid), FP, P, c_int, c_int, c_int, FP, c_float, c_int, c_float,
                                  P, P]),
    'srf_alpha_pool_threshold': (c_int, [P, c_int, c_int, c_int, c_float, P, P, P]),
    'srf_resample_grid': (c_int, [P, c_int, c_int, c_int, P, c_int, c_int, P]),
    'srf_crop_grid': (c_int, [P, c_int, c_int, c_int, c_int, c_int, P, c_int, c_int, P]),
    'srf_compact_workspace_size': (c_size_t, [c_int64]),
    'srf_compact': (c_int, [P, c_int64, P, P, P, c_size_t, P]),
    'srf_compact_noalloc': (c_int, [P, c_int64, P, P, P]),
    'srf_threshold_mask': (c_int, [P, c_int64, c_float, P, P]),
    'srf_gather_rows': (c_int, [P, P, c_int64, P, P, c_int64, c_int, c_int, P]),
    'srf_scatter_rows': (c_int, [P, c_int64, P, P, P, c_int64, c_int, P]),
    'srf_density_activation': (c_int, [P, c_int64, P, P, P, c_int64, c_int, c_float, P]),
    'srf_density_activation_backward': (c_int, [P, P, c_int64, P, P, P, c_int64, c_int, c_float, P]),
    'srf_tensorf_renderer_workspace_size': (c_size_t, [ctypes.POINTER(RendererDesc), c_int64, c_int, c_int]),
    'srf_tensorf_renderer_forward': (c_int, [ctypes.POINTER(RendererDesc), ctypes.POINTER(P), P, P, c_int64, P, c_int,
                                             c_int, P, c_size_t, P, P]),
    'srf_tensorf_renderer_backward': (c_int, [ctypes.POINTER(RendererDesc), ctypes.POINTER(P), P, P, c_int64,
                                              ctypes.POINTER(P), P, c_int, P, c_size_t, P, P]),
    'srf_linear_forward': (c_int, [P, c_int, P, c_int, P, P, c_int64, P, c_int, c_int, c_int, P]),
    'srf_linear_backward': (c_int, [P, c_int, P, P, P, c_int, P, c_int, P, c_int, P, P, c_int64, P, c_int, c_int,
                                    c_int, c_int, P]),
    'srf_positional_encoding_backward': (c_int, [P, P, P, c_int, c_int64, P, c_int, c_int, P]),
    'srf_rgb_depth_loss': (c_int, [P, P, P, P, P, c_int, c_int, c_float, P, P, P, P]),
    'srf_adam_step': (c_int, [P, P, P, P, c_int64, c_float, c_float, c_float, c_float, c_float, c_int, P, P, P]),
    'srf_counter_add': (c_int, [P, c_int, P, P]),
    'srf_depth_mse_loss': (c_int, [P, P, P, c_int, c_float, c_int, P, P, P, P]),
    'srf_mass_concentration_loss': (c_int, [P, c_int, c_int, c_int, P, c_float, P, P, P]),
    'srf_depth_reprojection_masks': (c_int, [P, P, P, P, P, c_int, P, c_int, P, P, c_int, c_int, c_int, c_int, c_int,
                                             c_float, P, P, P]),
    'srf_coarse_fine_reprojection_masks': (c_int, [P, P, P, P, P, c_int, P, c_int, P, P, c_int, c_int, c_int, c_int, c_int,
                                             c_float, P, P, P]),
    'srf_ray_points': (c_int, [P, P, P, c_int, c_int, P, P]),
    'srf_batch_assemble': (c_int, [P, P, P, c_int, c_int64, c_int64, c_int, ctypes.c_uint64, P, P, P, c_int, P, P, P, P, P, P]),
    'srf_uniforms': (c_int, [P, c_int64, ctypes.c_uint64, P, c_int, P]),
    'srf_tv_loss': (c_int, [ctypes.POINTER(TvComponent), c_int, c_float, P, P, P]),
    'srf_autotune_enable': (c_int, [c_int]),
    'srf_tensorf_basis_adjoint_path': (c_int, [c_int]),
    'srf_nerf_mlp_fused_path': (c_int, [c_int]),
    'srf_autotune_count': (c_int, []),
    'srf_autotune_entry': (c_int, [c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int64), ctypes.POINTER(c_int64),
                                   ctypes.POINTER(c_int64), ctypes.POINTER(c_int)]),
    'srf_autotune_set': (c_int, [c_int, c_int64, c_int64, c_int64, c_int]),
    'srf_autotune_clear': (c_int, []),
    'srf_adam_multi_step': (c_int, [ctypes.POINTER(AdamTensor), c_int, c_float, c_float, c_float, c_float, c_int, P,
                                    P, P]),
    'srf_launch_count': (c_int64, []),
}


def exported_symbols():
    """Names of every function the C header declares (used by the ABI test)."""
    return sorted(_SIGS)


_lib = None


def load():
    """Load the shared library (once); raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f'srf_gb300 CUDA library not built: {LIB_PATH} is missing '
                           '(run `python -m simple_rf_gb300.build`); there is no CPU fallback')
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    _tuner_from_env()
    return lib


def _tuner_from_env():
    """SRF_AUTOTUNE_TABLE=path preloads the tile-shape tuner's choices from a JSON
    table (autotune.save's format) when the file exists; SRF_AUTOTUNE_SAVE=path
    writes the table at exit.  A profiler replays and slows every launch, so a
    profiled process should start from the choices of an unprofiled run."""
    table, save = os.environ.get('SRF_AUTOTUNE_TABLE'), os.environ.get('SRF_AUTOTUNE_SAVE')
    if not (table or save):
        return
    from . import autotune
    if table and os.path.exists(table):
        autotune.load(table)
    if save:
        import atexit
        atexit.register(autotune.save, save)


def new_stream(device):
    """A CUDA stream of its own on ``device`` (srf_stream_create), as a torch
    stream; released when the returned object is collected.  Torch's pooled
    streams can alias one another (and the stream a CUDA graph is captured on),
    which would serialise stages meant to run concurrently."""
    import weakref
    import torch
    lib = load()
    ptr = P()
    with torch.cuda.device(device):
        check(lib.srf_stream_create(ctypes.byref(ptr)), 'srf_stream_create')
    st = torch.cuda.ExternalStream(ptr.value, device=device)
    fin = weakref.finalize(st, lib.srf_stream_destroy, P(ptr.value))
    # not at interpreter exit: tensors that recorded this stream can still be freed
    # after the exit finalizers ran, and the caching allocator then records an event
    # on the stream; the process's teardown releases it instead
    fin.atexit = False
    return st


def check(status, what=''):
    if status != 0:
        lib = load()
        msg = lib.srf_status_string(status).decode()
        if status == 5:
            msg += ' (' + lib.srf_last_cuda_error().decode() + ')'
        raise RuntimeError(f'{what}: {msg}')


def call(name, *args):
    """Call ``name`` and raise RuntimeError on a non-zero status."""
    lib = load()
    check(getattr(lib, name)(*args), name)


def host_floats(vals):
    arr = (ctypes.c_float * len(vals))(*[float(v) for v in vals])
    return arr
