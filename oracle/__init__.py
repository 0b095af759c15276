"""Oracle for cmpy_gb300 — TEST INFRASTRUCTURE ONLY.

Nothing in the product (``cmpy_gb300``) imports this package. It is used by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` as the checker.

* ``ed_oracle`` — a numpy/scipy restatement of the reference's hot path (sector
  enumeration, COO projectors, triplet matvec, dense eigh, thermal Lehmann Green's function,
  c^dag/c), each function citing the reference file:line it follows. It is pinned against
  golden vectors produced by the unmodified reference (``tests/golden/``).
* ``refshim`` — imports the unmodified reference (cmpy) from a source checkout with stub
  modules for its missing optional dependencies (numba, matplotlib, colorcet, gftool,
  lattpy). Only ``tests/golden/make_golden.py`` uses it, in a container that has the
  reference checkout; it never runs on the GPU machine.
"""
