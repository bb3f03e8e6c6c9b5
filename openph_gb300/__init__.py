"""openph_gb300 — GB300-native Z/2 boundary-matrix reduction (pms, and the
standard, twist and row variants) behind the reference OpenPH interface.

* :func:`ph` / :func:`openph` — the reference's MEX call and MATLAB wrapper.
* :class:`Context` — the context-based C API (0-based CSC, batches, device
  buffers).
* :class:`Server` — continuous-batching reduction server.
* :mod:`openph_gb300.complexes` — boundary matrices and seeded generators.

The reductions run only on the GPU through ``libopenph_gb300.so``.
"""
from .api import ALGORITHMS, Context, OphError, Server, ph, openph, status_string  # noqa: F401
from .complexes import BoundaryMatrix  # noqa: F401
