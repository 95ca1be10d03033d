"""A script that keeps a TensoRF training step (and the library's side streams)
alive until the interpreter exits must exit cleanly: the side streams the
library creates are not destroyed by the exit finalizers while tensors that
recorded them are still to be freed."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

SCRIPT = r'''
import torch
from simple_rf_gb300 import build as b
b.build()
from simple_rf_gb300.bench_tensorf import make_models, synthetic_rays
from simple_rf_gb300.tensorf_step import TensorfTrainStep
dev = torch.device('cuda')
models = make_models(dev, precision='fp16', grids=(64, 32))
st = TensorfTrainStep(models)
batch = synthetic_rays(2048, 1, dev)
st.step(*batch)
torch.cuda.synchronize()
print('stepped')
'''


def test_script_with_live_step_exits_cleanly():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, PYTHONPATH=root + os.pathsep + os.environ.get('PYTHONPATH', ''))
    r = subprocess.run([sys.executable, '-c', SCRIPT], cwd=root, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and 'stepped' in r.stdout, (r.returncode, r.stdout[-2000:], r.stderr[-2000:])
