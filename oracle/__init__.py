"""CPU oracle for the Simple-RF rendering hot path -- TEST INFRASTRUCTURE ONLY.

This package is a numpy restatement of the reference's rendering algorithm
(Simple-NeRF ``src/models/SimpleNeRF17.py`` and Simple-TensoRF
``src/models/SimpleTensoRF09.py``), forward and hand-derived backward, in any
float dtype (float32 for the 1e-5 parity bar, float64 for error statements).

It is the checker, never the product: only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py`` (its ``cpu_baseline`` leg and ``--impl reference`` arm) may
import it.  The product path (``simple_rf_gb300``) never imports this package.

Parity pinning: the restatement is checked against golden vectors produced by
running the reference's own model code (``tests/golden/make_golden.py``), see
``tests/test_oracle_golden.py``.
"""
