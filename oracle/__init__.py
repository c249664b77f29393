"""CPU oracle for the qTorch contraction path — TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of
``bench.py`` may import this package, and only as the checker: the product
(``qtorch_gb300``) never calls it and has no CPU fallback.

* ``port``: ctypes binding of ``qt_oracle.c`` (plain C restatement of
  src/Network.h:876-971 ContractIndices, src/Network.h:715-864 ContractNodes,
  the QASM parser src/Network.h:246-707 and the gate tables src/Node.h:197-898).
* ``qaoa_terms``: restatement of the MaxCut light-cone term generator
  (src/maxcut.h:31-233, src/maxcut.cpp:166-190).

Parity of the port itself is pinned by golden fixtures produced by the
unmodified reference headers (``oracle/_ref``; see ``tests/golden/make_golden.py``).
"""
from . import port  # noqa: F401
from . import qaoa_terms  # noqa: F401
