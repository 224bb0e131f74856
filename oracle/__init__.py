"""CPU oracle for the bond-based peridynamics time step (TEST INFRASTRUCTURE).

This package is test infrastructure only.  It is imported by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` as the
checker, never by the product package ``probabilistic_peridynamics_gb300``.

Contents
--------
``cl_step``      NumPy restatement of PeriPy's OpenCL step
                 (``peripy/cl/peridynamics.cl`` bond_force1..4 and damage,
                 ``peripy/cl/euler.cl``, ``euler_cromer.cl``,
                 ``velocity_verlet.cl``), including the exact pairwise
                 tree-reduction order of the work-group reduction, so that its
                 FP64 results are bit-reproducible.
``pp_oracle.c``  The same restatement in plain C (``-ffp-contract=off``) with
                 an OpenMP loop over nodes, for larger lattices and for the
                 timed CPU baseline when the compiled reference is absent.
``cref``         ctypes loader for ``pp_oracle.c``.
``ref``          Loader for the reference's own Cython CPU step compiled from
                 the reference sources into ``oracle/_ref`` by
                 ``oracle/build_ref.py``.

Parity is pinned against the reference's golden vectors
(``peripy/test/data/expected_*``) through the fixtures in ``tests/golden``.
"""
