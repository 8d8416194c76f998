"""CPU oracle for the hyperelastic finite-volume step (test infrastructure only).

This package is the oracle: a CPU restatement of BlackSiberian/HyperelasticSolver's
explicit first-order finite-volume step. Only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py`` (its ``cpu_baseline`` leg and ``--impl reference`` arm) may import it,
and only as the checker or as the timed CPU restatement of the reference. The GPU
product in ``hyperelasticsolver_gb300`` never imports it.

Parity status: unpinned against an execution of the reference (Julia is not
installed, and the reference has no tests or golden vectors). The C++ restatement
(``hyp_oracle.hpp``) is cross-checked against physics known-answer tests, LAPACK
eigenvalues and the independent transliteration in ``literal.py``.
"""
from .pyoracle import *  # noqa: F401,F403
