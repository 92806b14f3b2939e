"""CPU oracle for the Liouville-space propagation path (test infrastructure only).

This package is a plain NumPy/SciPy restatement of the reference algorithm
(whaley-group-berkeley/qspectra).  It exists to CHECK the CUDA path and to time
the CPU baseline; it is never imported by the product package
``qspectra_gb300``.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg use it.

Parity is pinned: ``tests/test_oracle_golden.py`` checks every function here
against fixtures in ``tests/golden/`` that ``tests/golden/make_golden.py``
generated by importing and running the reference itself.
"""
from .restatement import *  # noqa: F401,F403
