"""CPU oracle for the CP-ALS / Tucker-HOOI path (TEST INFRASTRUCTURE ONLY).

This package restates, in plain NumPy, the algorithms of TensorLy 0.9.0 that
the GB300 library replaces.  It exists to check the CUDA path, never to be
the CUDA path: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` may import it.  The product package
``tensorly_gb300`` never imports anything from here and fails loudly when its
CUDA library is missing.

Parity of this restatement with the reference is pinned by
``tests/golden/`` (fixtures generated by running the reference itself, see
``tests/golden/make_golden.py``) and checked by ``tests/test_oracle_golden.py``.
"""

from .tensorly_oracle import *  # noqa: F401,F403
