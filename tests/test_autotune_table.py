"""The tuning table's host API (no kernel launches): entries set, listed, saved,
preloaded and cleared."""
import os

from simple_rf_gb300 import autotune


def test_table_round_trip(tmp_path):
    autotune.clear()
    from simple_rf_gb300 import _lib
    lib = _lib.load()
    assert lib.srf_autotune_set(1, 256, 4, 0, 1) == 0
    assert lib.srf_autotune_set(3, 48, 48, 48, 2) == 0
    assert lib.srf_autotune_set(1, 256, 4, 0, 0) == 0          # overwrite
    assert lib.srf_autotune_set(2, 144, 192, 0, -1) != 0        # negative choice rejected
    t = {(e['site'], e['key']): e['choice'] for e in autotune.table()}
    assert t == {(1, (256, 4, 0)): 0, (3, (48, 48, 48)): 2}
    path = os.path.join(tmp_path, 'tune.json')
    autotune.save(path)
    autotune.clear()
    assert autotune.table() == []
    autotune.load(path)
    assert {(e['site'], e['key']): e['choice'] for e in autotune.table()} == t
    autotune.clear()


def test_table_preloaded_and_saved_through_the_environment(tmp_path):
    """SRF_AUTOTUNE_TABLE preloads a saved table when the library loads;
    SRF_AUTOTUNE_SAVE writes the process's table at exit (how a profiled run
    starts from an unprofiled run's choices)."""
    import json
    import subprocess
    import sys
    src = os.path.join(tmp_path, 'in.json')
    dst = os.path.join(tmp_path, 'out.json')
    with open(src, 'w') as f:
        json.dump([{'site': 1, 'key': [256, 4, 0], 'choice': 1}], f)
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ('from simple_rf_gb300 import _lib, autotune; _lib.load(); '
            'print([(e["site"], e["key"], e["choice"]) for e in autotune.table()])')
    env = dict(os.environ, SRF_AUTOTUNE_TABLE=src, SRF_AUTOTUNE_SAVE=dst, PYTHONPATH=repo)
    out = subprocess.run([sys.executable, '-c', code], env=env, capture_output=True, text=True, check=True, cwd=repo)
    assert out.stdout.strip() == '[(1, (256, 4, 0), 1)]', out.stdout + out.stderr
    with open(dst) as f:
        saved = json.load(f)
    assert [(e['site'], tuple(e['key']), e['choice']) for e in saved] == [(1, (256, 4, 0), 1)]
