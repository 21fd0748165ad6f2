"""CPU oracle for the autojax interferometer inversion — TEST INFRASTRUCTURE ONLY.

This package restates, in plain NumPy, the algorithm of the reference
implementation (``src/autojax/numba.py`` and, for the preload variant,
``src/autojax/original.py`` of ickc/python-autojax).  Every function cites the
reference lines it follows.

It is the checker, never the product:

* only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
  ``--impl reference`` legs of ``bench.py`` may import it;
* the GPU package ``autojax_gb300`` never imports it and has no CPU fallback.

Pinning: ``tests/golden/make_golden.py`` imports the reference itself (with a
pass-through ``numba`` shim, since numba is not installed) and writes its
outputs as fixtures; ``tests/test_oracle_golden.py`` checks this restatement
against those fixtures.  The adjoint in :mod:`oracle.adjoint` has no reference
counterpart (the reference has no gradient code); it is pinned by central
finite differences of the pinned log-evidence instead.
"""

from . import numpy_port  # noqa: F401
