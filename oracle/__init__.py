"""CPU oracle for the nodal DC path -- TEST INFRASTRUCTURE ONLY.

This package restates, in numpy/scipy, the reference's 3D nodal DC-resistivity
algorithm (``simpeg/electromagnetics/static/resistivity/simulation.py:100-263``
and ``:483-670``) together with the ``discretize`` TensorMesh operators it calls
(restated from their mathematical definitions, see ``operators.py``), solved
with SciPy SuperLU, which is what the reference's default ``SolverLU`` wraps
(``simpeg/utils/solver_utils.py:39-44``); the induced-polarization nodal
simulation on top of it (``ip3d.py``, after
``simpeg/electromagnetics/static/induced_polarization/simulation.py:15-167``).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference arm may import it, and only as the checker or the timed CPU
baseline.  Nothing in ``simpeg_gb300`` imports it.

Parity status: the restated ``discretize`` operators are pinned by the
reference's own tests (analytic half-space < 5 % rms, adjoint identity, Taylor
derivative order, custom-surface bit-equality, whole-space multipole fields
< 10 %, IP linearised-DC forward and adjoint; see ``tests/test_oracle.py``) and
by hand-checked tiny cases.  No golden vector from ``discretize`` itself exists
in the reference, so entry-wise parity with ``discretize`` is unpinned.
"""
