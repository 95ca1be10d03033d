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
