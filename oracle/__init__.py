"""CPU oracle for the flow-map -> FTLE -> ridge path.

TEST INFRASTRUCTURE ONLY: a plain-C restatement of the reference NumbaCS
algorithms (see ``oracle.c`` for the reference files and the third-party
algorithms it follows).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this package; the product library
``numbacs_gb300`` never does.
"""
from .oracle import *  # noqa: F401,F403
