"""CPU oracle for the jsolver_gb300 CUDA solver — test infrastructure, not product code.

A restatement of davef96/jsolver's algorithm (NumPy: ``mg2d``, ``mg3d``; C/OpenMP:
``jmg_oracle.c``) used only to check and to time against. The product package never
imports this package; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` do.
"""
