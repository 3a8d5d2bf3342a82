"""CPU oracle for the TransiFlow finite-volume hot path.

TEST INFRASTRUCTURE ONLY.  This package is the checker, never the product:
only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline / reference
arm of ``bench.py`` may import it.  The ``transiflow_gb300`` package never
imports it and never falls back to it.

It restates, in vectorised NumPy, the reference algorithm of BIMAU/transiflow
1.0.1 for the path the GPU backend replaces:

* ``oracle.fvm``   -- coordinates, atoms, boundary folding, RHS and CSR
  Jacobian assembly (``transiflow/Discretization.py``,
  ``transiflow/BoundaryConditions.py``, ``transiflow/CrsMatrix.py``,
  ``transiflow/utils.py``), keeping the reference's floating-point operation
  order so results agree bit for bit;
* ``oracle.solve`` -- the SciPy backend's direct solve: pressure gauge,
  bordering and SuperLU (``transiflow/interface/SciPy.py``).  The
  factorisation itself is SciPy's ``splu`` exactly as the reference calls it.

Parity of this restatement is pinned against the reference's own golden files
(``tests/data/*_4x4x4.txt``) and against fixtures generated by running the
reference (``tests/golden/make_golden.py``).
"""
