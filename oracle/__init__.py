"""CPU FP64 oracle for the SPECTRAX Hermite-Fourier right-hand side and its steppers.

TEST INFRASTRUCTURE ONLY. Nothing in the ``spectrax_gb300`` product path imports,
links or executes this package; only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline / reference arm use it, and only as the checker.

Parity status
-------------
* RHS (``oracle.rhs``), tables (``oracle.tables``) and energies (``oracle.diag``):
  pinned.  ``tests/golden/make_golden.py`` executes the reference's own
  ``spectrax/_simulation.py``, ``spectrax/_model.py``, ``spectrax/_initialization.py``
  and ``spectrax/_diagnostics.py`` with a NumPy stand-in for ``jax.numpy`` (JAX is
  not installable in this container) and stores the outputs as fixtures; the
  oracle is checked against them to 1e-13 in ``tests/test_oracle_golden.py``.
  What the stand-in cannot show is XLA's own FFT rounding (FP64, ~1e-16) and how
  XLA folds ``fftfreq`` for the 2/3 mask (see ``oracle.rhs.centered_cutoff``).
* Dopri8 (``oracle.dopri8``): the Prince-Dormand RK8(7)13M tableau is pinned by
  its order conditions (all 200 trees to order 8 for the solution weights, all
  85 trees to order 7 for the embedded weights).  Trajectory parity against
  Diffrax itself is UNPINNED: Diffrax is not installable here.
* Implicit midpoint (``oracle.midpoint``): UNPINNED against the reference (needs
  Diffrax and ``jax.linearize``); checked for consistency only.
"""
