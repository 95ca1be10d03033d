"""Build the srf_gb300 CUDA library in-tree for sm_103a.

    python -m simple_rf_gb300.build          # or simple_rf_gb300.build.build()

Each ``csrc/*.cu`` compiles in parallel to ``_build/*.o`` (one ``-gencode``,
``-lineinfo``) and links into ``simple_rf_gb300/libsrf_gb300.so``.  Objects are
rebuilt only when a source or header is newer.  No cmake, no torch headers: the
library's interface is the plain C ABI in ``include/srf_gb300.h``.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, 'csrc')
OUT_DIR = os.path.join(PKG, '_build')
LIB = os.path.join(PKG, 'libsrf_gb300.so')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
COMMON = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr',
          '-I' + os.path.join(REPO, 'include')]
# Per-file flags: the sampling and compositing formulas (the NDC depth
# conversion amplifies rounding near z = 1) must round like separate torch ops.
EXTRA = {'sampling.cu': ['-fmad=false'], 'composite.cu': ['-fmad=false'], 'vm.cu': ['-fmad=false'],
         'maintenance.cu': ['-fmad=false']}


def _nvcc():
    for cand in (os.environ.get('NVCC'), '/usr/local/cuda/bin/nvcc', 'nvcc'):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return 'nvcc'


def _newest_header():
    hs = glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(CSRC, '*.h')) + \
        glob.glob(os.path.join(REPO, 'include', '*.h'))
    return max([os.path.getmtime(h) for h in hs] or [0])


def _compile(src, verbose):
    name = os.path.basename(src)
    obj = os.path.join(OUT_DIR, name[:-3] + '.o')
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _newest_header()):
        return obj
    cmd = [_nvcc()] + ARCH + COMMON + EXTRA.get(name, []) + ['-c', src, '-o', obj]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f'nvcc failed for {name}:\n{r.stdout}\n{r.stderr}')
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose=False):
    """Compile every CUDA source and link the shared library; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, '*.cu')))
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc()] + ARCH + ['-shared', '-o', LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f'link failed:\n{r.stdout}\n{r.stderr}')
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv))
