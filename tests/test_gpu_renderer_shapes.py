"""The 16-bit TensoRF renderer (srf_tensorf_renderer_*) over shapes and row counts
beyond the benchmark model, through every path: the basis forward as the TF32
tensor-core pass or the SIMT pass (the tuner's choices 5 and 0), the basis adjoint
on the tensor cores or the fused SIMT pass (srf_tensorf_basis_adjoint_path; the
tensor-core adjoint needs C % 16 == 0, so C = 36 and C = 100 take the SIMT pass
either way).  Shapes: (C components, F features, U units, features PE, views PE,
view-dependent); rows 1, 129 (a partial second tile) and 5000.

Against the float64 oracle (renderer_forward / renderer_backward): rgb within 2e-3
max-abs on every path; d_feats and every parameter gradient within 0.1 relative L2
(a check for layout or sign errors, which give errors of order 1: the FP16 layers'
roundings flip ReLU masks of near-zero pre-activations of these random renderers,
a few percent on small row counts).  Between paths on the same forward: the
tensor-core and SIMT adjoints give d_feats within 3e-3 relative L2 (TF32 products),
dWb within 1e-4 and every other gradient within 1e-5; the four combinations agree
on rgb within 1e-3 max-abs."""
import numpy as np
import pytest
import torch

from oracle import tensorf as ot

pytestmark = pytest.mark.gpu
DEV = 'cuda'

SHAPES = [(144, 27, 128, 2, 2, 1), (48, 12, 128, 2, 2, 1), (96, 27, 256, 1, 4, 1), (16, 8, 128, 0, 0, 0),
          (256, 32, 128, 2, 2, 1), (36, 9, 128, 2, 2, 1), (100, 20, 128, 3, 1, 1)]


@pytest.fixture(scope='module', autouse=True)
def built():
    from simple_rf_gb300 import build as b
    b.build()


def _k1p(F, lf, lv, view):
    bw = (F + 7) // 8 * 8
    v0 = bw * (2 * lf + 1)
    return (v0 + (3 * (2 * lv + 1) if view else 0) + 63) // 64 * 64


@pytest.mark.parametrize('m', [1, 129, 5000])
@pytest.mark.parametrize('shape', SHAPES)
def test_renderer_paths_against_oracle(shape, m):
    from simple_rf_gb300 import _lib, autotune, tensorf as T
    C, F, U, lf, lv, view = shape
    spec = ot.RendererSpec(features_dim=F, features_pe=lf, views_pe=lv, units=U, use_view_dirs=bool(view))
    rng = np.random.default_rng(C + F + m)
    shapes = spec.param_shapes(C)
    p = {k: (rng.standard_normal(sh) * (sh[1] ** -0.5 if len(sh) == 2 else 0.05)).astype(np.float32)
         for k, sh in shapes.items()}
    f = (rng.standard_normal((m, C)) * 0.3).astype(np.float32)
    v = rng.standard_normal((m, 3)).astype(np.float32)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    g = rng.standard_normal((m, 3)).astype(np.float32)
    p64 = {k: x.astype(np.float64) for k, x in p.items()}
    rgb64, cache = ot.renderer_forward(p64, spec, f.astype(np.float64), v.astype(np.float64))
    g64, df64 = ot.renderer_backward(p64, spec, cache, g.astype(np.float64))
    desc = _lib.RendererDesc(C, F, U, lf, lv, view)
    lib = _lib.load()
    key = (C, _k1p(F, lf, lv, view), 0)
    rgbs, grads = {}, {}
    try:
        autotune.enable(False)
        for fwd in (0, 5):
            for adj in (0, 1):
                _lib.check(lib.srf_autotune_set(2, *key, fwd), 'srf_autotune_set')
                _lib.check(lib.srf_tensorf_basis_adjoint_path(adj), 'srf_tensorf_basis_adjoint_path')
                params = [torch.from_numpy(p[k]).to(DEV).requires_grad_(True) for k in shapes]
                feats = torch.from_numpy(f).to(DEV).requires_grad_(True)
                rgb = T.renderer_tc(desc, _lib.SRF_PRECISION_FP16, feats, torch.from_numpy(v).to(DEV) if view else None,
                                    params)
                rgb.backward(torch.from_numpy(g).to(DEV))
                torch.cuda.synchronize()
                tag = f'fwd{fwd}_adj{adj}'
                got = rgb.detach().cpu().numpy()
                rgbs[tag] = got
                err = float(np.abs(got - rgb64).max())
                assert err < 2e-3, (tag, err)
                gr = {'d_feats': feats.grad.cpu().numpy()}
                gr.update({k: t.grad.cpu().numpy() for k, t in zip(shapes, params)})
                grads[tag] = gr
                rel = {k: float(np.linalg.norm(x - (df64 if k == 'd_feats' else g64[k])) /
                                max(np.linalg.norm(df64 if k == 'd_feats' else g64[k]), 1e-30)) for k, x in gr.items()}
                worst = max(rel.items(), key=lambda kv: kv[1])
                assert worst[1] < 0.1, (tag, worst, rel)
    finally:
        lib.srf_tensorf_basis_adjoint_path(1)
        autotune.clear()
        autotune.enable(True)
    tags = list(rgbs)
    for t in tags[1:]:
        assert float(np.abs(rgbs[t] - rgbs[tags[0]]).max()) < 1e-3, (t, tags[0])
    for fwd in (0, 5):
        simt, tc = grads[f'fwd{fwd}_adj0'], grads[f'fwd{fwd}_adj1']
        for k in simt:
            bar = 3e-3 if k == 'd_feats' else (1e-4 if k == 'basis_matrix_color.weight' else 1e-5)
            rel = float(np.linalg.norm(tc[k] - simt[k]) / max(np.linalg.norm(simt[k]), 1e-30))
            assert rel < bar, (fwd, k, rel)
